// pt_engine.cu -- the PT-ICM engine for sm_103a.
//
// One persistent kernel runs `nsteps` parallel-tempering steps for a batch of
// instances.  A step is, as in the reference's solve loop
// (src/solver.cc:67-127):
//   1. Metropolis sweeps of every replica        (src/replica.cc:5-38)
//   2. replica exchange, chains*(nt-1) attempts  (src/replica_exchange.cc:5-100)
//   3. isoenergetic cluster moves on the nc coldest temperatures
//                                                (src/icm.cc:8-215)
//
// Layout: every replica of an instance lives in shared memory of the block
// that owns it (int8 spins, int32 local fields f_i = sum_j J_ij s_j), the
// adjacency is staged into shared memory by bulk (TMA) copies, and exchange
// permutes the slot->replica map instead of moving spins.  A block owns `rpc`
// replicas of one instance; `group` blocks share an instance and meet at a
// bounded grid barrier once per step (cooperative launch).
//
// Production sweeps visit the sites colour class by colour class (no two
// sites of a class are adjacent) with Philox uniforms compared against
// per-temperature integer thresholds ceil(exp(-beta*dE) * 2^32), computed on
// the host in FP64.  The replay variant visits sites in the reference's
// sequential order and consumes a recorded uniform stream with FP64
// exp(-beta*dE) tables, reproducing the reference bit for bit.
#include <algorithm>
#include <atomic>
#include <cstdint>
#include <cstdio>

#include "pticm_device.cuh"
#include "pticm_engine.h"

namespace pticm {

template <typename T>
__device__ __forceinline__ T* sm_ptr(uint8_t* base, uint32_t off) {
    return reinterpret_cast<T*>(base + off);
}

// Thread-0 phase timers (clock64), enabled by EngineArgs::prof.
struct Prof {
    bool on;
    long long mark, sub;
    long long* c;   // PROF_PHASES counters in shared memory (thread 0 only)
    __device__ __forceinline__ void init(bool enable, long long* store) {
        on = enable;
        c = store;
        mark = sub = enable ? clock64() : 0;
        if (enable)
            for (int q = 0; q < PROF_PHASES; q++) c[q] = 0;
    }
    __device__ __forceinline__ void tick(int slot) {
        if (on) { const long long t = clock64(); c[slot] += t - mark; mark = t; sub = t; }
    }
    __device__ __forceinline__ void subtick(int slot) {
        if (on) { const long long t = clock64(); c[slot] += t - sub; sub = t; }
    }
};

// ------------------------------------------------------------ union-find
// Concurrent union-find in shared memory: roots are hooked larger-under-
// smaller with CAS (parent indices strictly decrease, so no cycle forms) and
// finds halve paths.  Loops are capped; -1 / false report the cap.
__device__ __forceinline__ int uf_find(volatile int* parent, int x) {
    for (int it = 0; it < (1 << 20); it++) {
        const int p = parent[x];
        if (p == x) return x;
        const int gp = parent[p];
        if (gp == p) return p;
        parent[x] = gp;
        x = gp;
    }
    return -1;
}

__device__ __forceinline__ bool uf_unite(int* parent, int a, int b) {
    volatile int* vp = parent;
    for (int it = 0; it < (1 << 20); it++) {
        a = uf_find(vp, a);
        b = uf_find(vp, b);
        if (a < 0 || b < 0) return false;
        if (a == b) return true;
        if (a < b) { const int t = a; a = b; b = t; }
        if (atomicCAS(parent + a, a, b) == a) return true;
    }
    return false;
}

// ---------------------------------------------------------- team helpers
// An ICM "team" is either one warp (many pairs per block) or the whole block
// (one pair per block).  Block-wide reductions go through shared scratch.
// A block team reduces through three slots of four words, used in turn: a
// slot is reset by the reduction after the one that used it (whose barrier
// every reader of the slot has passed), so one barrier per reduction
// suffices.  Between teams all slots hold the identity (0, ~0, ~0, 0).
__device__ __forceinline__ void team_slot_reset(long long* acc, int slot) {
    unsigned long long* u = reinterpret_cast<unsigned long long*>(acc) + 4 * slot;
    u[0] = 0;
    u[1] = ~0ull;
    u[2] = ~0ull;
    u[3] = 0;
}

template <bool BLOCK>
struct Team {
    int tr, ts;                  // rank and size
    long long* acc;              // team scratch (shared, 12 words for a block team)
    int* ctl;                    // team scratch (shared): BFS queue tail, vote
    mutable int k = 0;           // reductions so far (the same in every thread)
    __device__ __forceinline__ void sync() const {
        if (BLOCK) __syncthreads(); else __syncwarp();
    }
    // (sum, min, min, sum) over the team
    __device__ __forceinline__ void reduce(long long& s0, unsigned long long& m1, unsigned long long& m2,
                                           long long& s3) const {
        for (int o = 16; o > 0; o >>= 1) {
            s0 += __shfl_xor_sync(0xffffffffu, s0, o);
            m1 = min(m1, __shfl_xor_sync(0xffffffffu, m1, o));
            m2 = min(m2, __shfl_xor_sync(0xffffffffu, m2, o));
            s3 += __shfl_xor_sync(0xffffffffu, s3, o);
        }
        if (!BLOCK) return;
        const int slot = k % 3;
        unsigned long long* u = reinterpret_cast<unsigned long long*>(acc) + 4 * slot;
        if ((threadIdx.x & 31) == 0) {
            atomicAdd(u + 0, (unsigned long long)s0);
            atomicMin(u + 1, m1);
            atomicMin(u + 2, m2);
            atomicAdd(u + 3, (unsigned long long)s3);
        }
        __syncthreads();
        s0 = (long long)u[0]; m1 = u[1]; m2 = u[2]; s3 = (long long)u[3];
        if (threadIdx.x == 0 && k > 0) team_slot_reset(acc, (k + 2) % 3);
        k++;
    }
    __device__ __forceinline__ void sum2(long long& a, long long& b) const {
        unsigned long long x = ~0ull, y = ~0ull;
        reduce(a, x, y, b);
    }
};

// 64-bit finaliser of splitmix64 (Steele, Lea, Flood, OOPSLA 2014): a
// bijective mixer giving independent-looking keys for consecutive inputs.
__device__ __forceinline__ unsigned long long mix64(unsigned long long z) {
    z = (z ^ (z >> 30)) * 0xBF58476D1CE4E5B9ull;
    z = (z ^ (z >> 27)) * 0x94D049BB133111EBull;
    return z ^ (z >> 31);
}

// Per-block view of the launch.
struct BlockCtx {
    InstanceDesc D;
    int rank, r0;
    const int32_t* row;
    const uint32_t* adj;
    int8_t* spin;
    int32_t* field;
    const int32_t* h;
    long long* E;
    uint32_t* slot;
    uint32_t* rslot;
    int32_t* tb;        // threshold row base of each local replica
};

// ICM team scratch: BFS queue / union-find parents (n ints), overlap flags
// (n bytes), visited bits (icm_team_bytes); a block team's overlap list (n
// ints) follows (icm_block_bytes of the shared-memory plan).
struct IcmScratch {
    int* queue;
    uint8_t* d;
    uint32_t* vis;
    int* list;          // block team only: overlap sites first, the others from the end
};

__device__ __forceinline__ IcmScratch icm_scratch(uint8_t* base, int n_pad) {
    IcmScratch X;
    X.queue = reinterpret_cast<int*>(base);
    X.d = base + (size_t)n_pad * 4;
    X.vis = reinterpret_cast<uint32_t*>(base + (size_t)n_pad * 5);
    X.list = reinterpret_cast<int*>(base + icm_team_bytes(n_pad));
    return X;
}

// Calls f(e) for every packed entry (col << 8 | uint8 J) of site i's
// neighbour list: a scalar head up to a 16-byte boundary, four entries per
// 16-byte load, a scalar tail (plain loads: the list may be staged in shared
// memory; a list that is not 16-byte aligned is walked entry by entry).
// For small bodies only (field gathers and pushes): the body is expanded
// several times, and a large one (union-find) costs more in instruction
// fetch than the wider loads save.
template <class F>
__device__ __forceinline__ void for_each_neighbour(const int32_t* row, const uint32_t* adj, int i, F&& f) {
    int a = row[i];
    const int e1 = row[i + 1];
    if ((reinterpret_cast<uintptr_t>(adj) & 15u) == 0) {
        for (; a < e1 && (a & 3); a++) f(adj[a]);
#pragma unroll 2
        for (; a + 4 <= e1; a += 4) {
            const uint4 q = *reinterpret_cast<const uint4*>(adj + a);
            f(q.x);
            f(q.y);
            f(q.z);
            f(q.w);
        }
    }
    for (; a < e1; a++) f(adj[a]);
}

// ------------------------------------------------------------------ ICM
// One cluster move on the pair (A, B) = (chain 2c, chain 2c+1) at slot k.
// The team computes the overlap (sites where A and B differ), the
// reference's global-flip rule (src/icm.cc:20-28: more than n/2 differing
// sites -> negate A), a seed uniform among differing sites (src/icm.cc:33;
// here the differing site with the smallest per-site random key, which is
// uniform), then finds the seed's cluster C of differing sites -- breadth-
// first, or by labelling the components of the whole overlap (src/icm.cc:
// 37-72 grows it depth-first; the cluster is the same set) -- and flips the
// smaller of C and the rest of the overlap in both replicas.  Fields are
// updated per flipped site (or recomputed when the set is large); energies
// change by -2 s_u h_u per flipped site plus -2 J s_u s_v per edge leaving
// the set (s_v equal in A and B), an exact integer update.  Members held by
// another block are read from the published copy and flipped by their own
// block, which finds the same set.
template <bool BLOCK, bool REPLAY, bool LS, bool GLINK = false>
__device__ int icm_pair(const EngineArgs& A, const BlockCtx& B, const Team<BLOCK>& team, int q,
                         int rA, int rB, unsigned long long step, int ls, const IcmScratch& X,
                         int where_err, Prof& P) {
    const InstanceDesc& D = B.D;
    const int n = D.n, npad = D.n_pad;
    // the block context lives in shared memory: its pointers and flags are
    // read once here, not at every use inside the passes' loops
    const int32_t* const brow = B.row;
    const uint32_t* const badj = B.adj;
    const int32_t* const bh = D.has_h ? B.h : nullptr;
    const bool has_h = bh != nullptr;
    const bool locA = rA >= B.r0 && rA < B.r0 + D.rpc;
    const bool locB = rB >= B.r0 && rB < B.r0 + D.rpc;
    const int parity = (int)(step & 1ull);
    const int8_t* pubA = A.spins_pub + parity * A.spins_pub_half + D.spin_off + (long long)rA * npad;
    const int8_t* pubB = A.spins_pub + parity * A.spins_pub_half + D.spin_off + (long long)rB * npad;
    int8_t* sA = locA ? B.spin + (rA - B.r0) * npad : nullptr;
    int8_t* sB = locB ? B.spin + (rB - B.r0) * npad : nullptr;
    // no stored fields in field_gather mode: field updates are skipped
    int32_t* fA = (locA && B.field) ? B.field + (rA - B.r0) * npad : nullptr;
    int32_t* fB = (locB && B.field) ? B.field + (rB - B.r0) * npad : nullptr;
    uint8_t* d = X.d;
    const int nwords = (n + 31) >> 5;
    if (threadIdx.x == 0) P.subtick(PROF_ICM_ENERGY);
    // a caller's seed for this pair (device numbering), or skip the pair
    int forced = -1;
    const bool exact = REPLAY || A.icm_exact != 0;
    if (!REPLAY && A.icm_force != nullptr) {
        const long long f = A.icm_force[q];
        if (f == -2) return 0;
        if (f >= (long long)n || f < -2) {
            if (team.tr == 0) dev_fail(A.status, A.abort_flag, DEV_BAD_INDEX, where_err + 5, q, f);
            return 0;
        }
        if (f >= 0) forced = A.perm[D.perm_off + f];
    }

    // overlap, its size, seed candidates among differing and equal sites
    unsigned long long r64 = 0;
    if (!REPLAY) {
        const uint4 rnd = philox4x32_10(make_uint4((uint32_t)q, (uint32_t)D.inst_id, (uint32_t)step,
                                                   (uint32_t)(step >> 32)), stream_key(A.seed, STREAM_ICM));
        r64 = ((unsigned long long)rnd.y << 32) | rnd.x;
    }
    long long cnt = 0, hs = 0;
    unsigned long long kd = ~0ull, ke = ~0ull;
    const int algo = D.icm_algo;
    auto overlap_site = [&](int i, int8_t a, int8_t b) {
        const bool di = a != b;
        d[i] = di;
        if (algo == ENGINE_ICM_UNION_FIND) X.queue[i] = i;   // union-find parents
        cnt += di;
        if (!REPLAY) {
            const unsigned long long key = (mix64(r64 + 0x9E3779B97F4A7C15ull * (unsigned long long)(i + 1)) &
                                            0xFFFFFFFF00000000ull) | (unsigned)i;
            if (di) kd = min(kd, key);
            else ke = min(ke, key);
        }
        if (has_h && locA) hs += (long long)bh[i] * a;
    };
    // a block team lists the overlap sites (from the front) and the others
    // (from the back), so that its later passes visit overlap sites only;
    // the counters are team.ctl[2..3], zero between pairs
    int* lst = X.list;
    auto append = [&](bool valid, bool di, int i) {
        const int lane = threadIdx.x & 31;
        const unsigned mf = __ballot_sync(0xffffffffu, valid && di);
        const unsigned mb = __ballot_sync(0xffffffffu, valid && !di);
        int f0 = 0, b0 = 0;
        if (lane == 0) {
            if (mf) f0 = atomicAdd(team.ctl + 2, __popc(mf));
            if (mb) b0 = atomicAdd(team.ctl + 3, __popc(mb));
        }
        f0 = __shfl_sync(0xffffffffu, f0, 0);
        b0 = __shfl_sync(0xffffffffu, b0, 0);
        const unsigned lt = (1u << lane) - 1u;
        const int pf = f0 + __popc(mf & lt), pb = n - 1 - b0 - __popc(mb & lt);
        if (valid && di && pf < n) lst[pf] = i;
        if (valid && !di && pb >= 0) lst[pb] = i;
    };
    if (BLOCK && LS) {
        // four sites per thread: one 32-bit word of each replica's spins (the
        // partner's from the published copy in L2, one load for all four),
        // the overlap flags stored as one word, and the sites appended to
        // the list with one warp scan and one atomic per warp and list
        // (rows are n_pad bytes, a multiple of 16: every word is aligned)
        const int lane = threadIdx.x & 31;
        const int nq = (n + 3) >> 2;
        // the next round's words are loaded before this round's are used
        // (a partner's words come from its published copy in L2)
        auto load_words = [&](int w, uint32_t& wa, uint32_t& wb) {
            wa = locA ? reinterpret_cast<const uint32_t*>(sA)[w] : __ldcg(reinterpret_cast<const unsigned int*>(pubA) + w);
            wb = locB ? reinterpret_cast<const uint32_t*>(sB)[w] : __ldcg(reinterpret_cast<const unsigned int*>(pubB) + w);
        };
        uint32_t na = 0, nb = 0;
        if (team.tr < nq) load_words(team.tr, na, nb);
        for (int w0 = 0; w0 < nq; w0 += team.ts) {
            const int w = w0 + team.tr;
            const bool have = w < nq;
            const uint32_t wa = na, wb = nb;
            if (w + team.ts < nq) load_words(w + team.ts, na, nb);
            uint32_t dw = 0;
            int fm = 0, bm = 0;
            if (have) {
#pragma unroll
                for (int j = 0; j < 4; j++) {
                    const int i = 4 * w + j;
                    if (i >= n) break;
                    const int8_t a = (int8_t)(wa >> (8 * j)), b = (int8_t)(wb >> (8 * j));
                    const bool di = a != b;
                    dw |= (uint32_t)di << (8 * j);
                    fm |= (int)di << j;
                    bm |= (int)!di << j;
                    cnt += di;
                    const unsigned long long key =
                        (mix64(r64 + 0x9E3779B97F4A7C15ull * (unsigned long long)(i + 1)) & 0xFFFFFFFF00000000ull) |
                        (unsigned)i;
                    if (di) kd = min(kd, key);
                    else ke = min(ke, key);
                    if (has_h && locA) hs += (long long)bh[i] * a;
                }
                reinterpret_cast<uint32_t*>(d)[w] = dw;
                if (algo == ENGINE_ICM_UNION_FIND)   // union-find parents
                    reinterpret_cast<int4*>(X.queue)[w] = make_int4(4 * w, 4 * w + 1, 4 * w + 2, 4 * w + 3);
            }
            // list positions: both counts packed in one int, one inclusive scan
            const int packed = __popc(fm) | (__popc(bm) << 16);
            int incl = packed;
#pragma unroll
            for (int o = 1; o < 32; o <<= 1) {
                const int v = __shfl_up_sync(0xffffffffu, incl, o);
                if (lane >= o) incl += v;
            }
            int base_f = 0, base_b = 0;
            if (lane == 31) {
                if (incl & 0xffff) base_f = atomicAdd(team.ctl + 2, incl & 0xffff);
                if (incl >> 16) base_b = atomicAdd(team.ctl + 3, incl >> 16);
            }
            base_f = __shfl_sync(0xffffffffu, base_f, 31);
            base_b = __shfl_sync(0xffffffffu, base_b, 31);
            const int excl = incl - packed;
            int pf = base_f + (excl & 0xffff), pb = n - 1 - (base_b + (excl >> 16));
#pragma unroll
            for (int j = 0; j < 4; j++) {
                if ((fm >> j) & 1) lst[pf++] = 4 * w + j;
                if ((bm >> j) & 1) lst[pb--] = 4 * w + j;
            }
        }
    } else {
        // two sites per round, both loaded first: the partner's spins come
        // from the published copy in L2 (the wide 1024-thread variants keep
        // this shorter code, which needs fewer registers)
        for (int base = 0; base < n; base += 2 * team.ts) {
            const int i = base + team.tr, i2 = i + team.ts;
            int8_t a = 0, b = 0, a2 = 0, b2 = 0;
            if (i < n) {
                a = locA ? sA[i] : ld_cg(pubA + i);
                b = locB ? sB[i] : ld_cg(pubB + i);
            }
            if (i2 < n) {
                a2 = locA ? sA[i2] : ld_cg(pubA + i2);
                b2 = locB ? sB[i2] : ld_cg(pubB + i2);
            }
            if (i < n) overlap_site(i, a, b);
            if (i2 < n) overlap_site(i2, a2, b2);
            if (BLOCK) {
                append(i < n, a != b, i);
                append(i2 < n, a2 != b2, i2);
            }
        }
    }
    if (algo == ENGINE_ICM_BFS)   // the visited bits of the breadth-first search
        for (int w = team.tr; w < nwords; w += team.ts) X.vis[w] = 0u;
    team.reduce(cnt, kd, ke, hs);
    const bool gflip = cnt > (long long)(n / 2);
    if (forced >= 0 && (d[forced] != 0) == gflip) {
        // a caller's seed must be a differing site after the global flip:
        // report it before any state changes (and clear the list counters)
        if (team.tr == 0) dev_fail(A.status, A.abort_flag, DEV_BAD_INDEX, where_err + 6, q, forced);
        if (BLOCK && team.tr == 0) { team.ctl[2] = 0; team.ctl[3] = 0; team.ctl[4] = 0; }
        team.sync();
        return 0;
    }
    // the overlap list of a block team: [l0, l0 + llen) of lst
    const int l0 = gflip ? (int)cnt : 0, llen = gflip ? n - (int)cnt : (int)cnt;
    auto for_overlap = [&](auto&& f) {
        if (BLOCK) {
            for (int t = team.tr; t < llen; t += team.ts) f(lst[l0 + t]);
        } else {
            for (int u = team.tr; u < n; u += team.ts)
                if (d[u]) f(u);
        }
    };
    long long dEa = 0, dEb = 0;
    if (gflip) {
        for (int i = team.tr; i < n; i += team.ts) {
            if (locA) { sA[i] = (int8_t)-sA[i]; if (fA) fA[i] = -fA[i]; }
            d[i] ^= 1;
        }
        cnt = n - cnt;
        if (team.tr == 0) dEa = -2 * hs;   // E(-s) = E(s) - 2 sum h s
        team.sync();
    }
    if (threadIdx.x == 0) P.subtick(PROF_ICM_DIFF);
    int seed = -1;
    if (REPLAY) {
        const long long idx = (long long)ls * D.nc + q;
        const long long traced = (idx < (long long)A.replay.n_icm) ? A.replay.icm_seed[idx] : -2;
        if ((traced < 0) != (cnt == 0)) {
            if (team.tr == 0) dev_fail(A.status, A.abort_flag, DEV_REPLAY_MISMATCH, where_err, idx, cnt);
            return 0;
        }
        if (cnt > 0) {
            if (traced >= n) {
                if (team.tr == 0) dev_fail(A.status, A.abort_flag, DEV_BAD_INDEX, where_err + 1, idx, traced);
                return 0;
            }
            seed = A.perm[D.perm_off + traced];
            if (!d[seed]) {
                if (team.tr == 0) dev_fail(A.status, A.abort_flag, DEV_REPLAY_MISMATCH, where_err + 2, idx, seed);
                return 0;
            }
        }
    } else if (cnt > 0) {
        seed = forced >= 0 ? forced : (int)((gflip ? ke : kd) & 0xFFFFFFFFull);
        if (seed < 0 || seed >= n) {
            if (team.tr == 0) dev_fail(A.status, A.abort_flag, DEV_BAD_INDEX, where_err + 4, q, seed);
            return 0;
        }
    }
    if (threadIdx.x == 0) P.subtick(PROF_ICM_SEED);
    bool absolute = false;   // energies set from scratch (large flipped sets)
    int swapped = 0;         // the flipped set was D\C (the chains hold each other's result)
    // a block team's union-find lists the sites it found outside the giant
    // component L in the free part of lst (S, at sbase); when the flipped set
    // lies in S it is taken from there: the sites of S whose final root is
    // (fast_eq) or is not (!fast_eq) fast_root
    bool fast = false, fast_eq = false;
    int fast_root = -1, ns = 0;
    const int sbase = l0 == 0 ? llen : 0;
    if (cnt > 0) {
        long long csize = 0;
        if (algo == ENGINE_ICM_BFS) {
            // breadth-first search from the seed; members of C get d = 2
            // (the visited bits make each site's claim unique)
            volatile int* vctl = team.ctl;
            if (team.tr == 0) {
                X.queue[0] = seed;
                X.vis[seed >> 5] |= 1u << (seed & 31);
                d[seed] = 2;
                vctl[1] = 1;
            }
            team.sync();
            const int lane = threadIdx.x & 31;
            int lo = 0;
            for (int level = 0; level <= n; level++) {
                const int hi = vctl[1];
                team.sync();
                if (lo == hi) break;
                for (int base = lo; base < hi; base += team.ts) {
                    const int idx = base + team.tr;
                    const bool have = idx < hi;
                    const int u = have ? X.queue[idx] : 0;
                    const int e0 = have ? brow[u] : 0;
                    const int deg = have ? brow[u + 1] - e0 : 0;
                    for (int k = 0; __any_sync(0xffffffffu, k < deg); k++) {
                        bool found = false;
                        int v = 0;
                        if (k < deg) {
                            v = (int)(badj[e0 + k] >> 8);
                            if (((volatile uint8_t*)d)[v] == 1) {
                                const uint32_t bit = 1u << (v & 31);
                                found = !(atomicOr(X.vis + (v >> 5), bit) & bit);
                            }
                        }
                        const unsigned m = __ballot_sync(0xffffffffu, found);
                        if (m) {
                            const int leader = __ffs(m) - 1;
                            int slot0 = 0;
                            if (lane == leader) slot0 = atomicAdd(team.ctl + 1, __popc(m));
                            slot0 = __shfl_sync(0xffffffffu, slot0, leader);
                            if (found) {
                                X.queue[slot0 + __popc(m & ((1u << lane) - 1u))] = v;
                                d[v] = 2;
                            }
                        }
                    }
                }
                team.sync();
                lo = hi;
            }
            csize = lo;
            if (threadIdx.x == 0) P.subtick(PROF_ICM_UNION);
        } else {
            // label the components of the whole overlap subgraph, then mark the
            // sites sharing the seed's label
            int* lab = X.queue;
            volatile int* vl = lab;
            bool ok = true;
            // (union-find parents were set with the overlap)
            if (algo != ENGINE_ICM_UNION_FIND) {
                for (int i = team.tr; i < n; i += team.ts) lab[i] = d[i] ? i : n;
                team.sync();
            }
            if (algo == ENGINE_ICM_UNION_FIND) {
                // Afforest (Sutton, Ben-Nun, Barak, IPDPS 2018): in two
                // rounds, link every overlap site to its r-th overlap
                // neighbour and compress the trees; take the most frequent
                // root of a sample as the large component L, then process the
                // full adjacency only of sites outside L.  An edge skipped at
                // an end in L is processed from its other end, unless that end
                // is in L too -- then both are already joined.
                // (GLINK: with the neighbour lists in device memory, a
                // thread scans four of its sites side by side, so that
                // their dependent loads overlap, then makes their unions)
                const bool glink = GLINK && BLOCK && !__isShared(badj);
                // (a block team's round 0 also finds each site's second
                // overlap neighbour and keeps it, by list position, in the
                // free part of the list -- S is listed there only later --
                // for round 1)
                int* const link1 = (BLOCK && (LS || GLINK)) ? lst + sbase : nullptr;
                for (int round = 0; round < 2; round++) {
                    if (round == 1 && link1 != nullptr) {
                        for (int t = team.tr; t < llen; t += 4 * team.ts) {
                            int u[4], tg[4];
#pragma unroll
                            for (int k = 0; k < 4; k++) {
                                const int tk = t + k * team.ts;
                                u[k] = tk < llen ? lst[l0 + tk] : -1;
                                tg[k] = tk < llen ? link1[tk] : -1;
                            }
#pragma unroll
                            for (int k = 0; k < 4; k++)
                                if (u[k] >= 0 && tg[k] >= 0) ok &= uf_unite(lab, u[k], tg[k]);
                        }
                    } else if (glink) {
                        for (int t = team.tr; t < llen; t += 4 * team.ts) {
                            int u[4], a[4], e[4], tg[4], k4[4];
#pragma unroll
                            for (int k = 0; k < 4; k++) {
                                const int tk = t + k * team.ts;
                                u[k] = tk < llen ? lst[l0 + tk] : -1;
                            }
#pragma unroll
                            for (int k = 0; k < 4; k++) {
                                a[k] = u[k] >= 0 ? brow[u[k]] : 0;
                                e[k] = u[k] >= 0 ? brow[u[k] + 1] : 0;
                            }
                            uint32_t v[4][4];
#pragma unroll
                            for (int k = 0; k < 4; k++)
#pragma unroll
                                for (int j = 0; j < 4; j++) v[k][j] = a[k] + j < e[k] ? badj[a[k] + j] : 0xFFFFFFFFu;
                            // the round-th overlap neighbour (tg) and, in
                            // round 0 with a place to keep it, the next (t1)
                            const int want = (round == 0 && link1 != nullptr) ? 2 : round + 1;
                            int t1[4];
#pragma unroll
                            for (int k = 0; k < 4; k++) {
                                tg[k] = -1;
                                t1[k] = -1;
                                k4[k] = 0;
#pragma unroll
                                for (int j = 0; j < 4; j++) {
                                    const bool on = v[k][j] != 0xFFFFFFFFu && d[v[k][j] >> 8];
                                    if (on && k4[k] < want) {
                                        if (k4[k] == round) tg[k] = (int)(v[k][j] >> 8);
                                        else if (k4[k] == round + 1) t1[k] = (int)(v[k][j] >> 8);
                                        k4[k]++;
                                    }
                                }
                            }
#pragma unroll
                            for (int k = 0; k < 4; k++) {
                                if (u[k] < 0) continue;
                                // the targets past the first four entries: four
                                // independent loads at a time
                                for (int aa = a[k] + 4; aa < e[k] && k4[k] < want; aa += 4) {
                                    uint32_t w4[4];
#pragma unroll
                                    for (int j = 0; j < 4; j++) w4[j] = aa + j < e[k] ? badj[aa + j] : 0xFFFFFFFFu;
#pragma unroll
                                    for (int j = 0; j < 4; j++) {
                                        const bool on = w4[j] != 0xFFFFFFFFu && d[w4[j] >> 8];
                                        if (on && k4[k] < want) {
                                            if (k4[k] == round) tg[k] = (int)(w4[j] >> 8);
                                            else if (k4[k] == round + 1) t1[k] = (int)(w4[j] >> 8);
                                            k4[k]++;
                                        }
                                    }
                                }
                                if (round == 0 && link1 != nullptr) link1[t + k * team.ts] = t1[k];
                                if (tg[k] >= 0) ok &= uf_unite(lab, u[k], tg[k]);
                            }
                        }
                    } else if (link1 != nullptr) {
                        // round 0 of a block team: the first two overlap
                        // neighbours, the list four entries at a time
                        for (int t = team.tr; t < llen; t += team.ts) {
                            const int u = lst[l0 + t];
                            int k = 0, tgt = -1, t1 = -1;
                            const int e1 = brow[u + 1];
                            for (int a = brow[u]; a < e1 && k < 2; a += 4) {
                                int v[4];
                                bool on[4];
#pragma unroll
                                for (int j = 0; j < 4; j++) v[j] = a + j < e1 ? (int)(badj[a + j] >> 8) : u;
#pragma unroll
                                for (int j = 0; j < 4; j++) on[j] = a + j < e1 && d[v[j]];
#pragma unroll
                                for (int j = 0; j < 4; j++)
                                    if (on[j] && k < 2) {
                                        if (k == 0) tgt = v[j];
                                        else t1 = v[j];
                                        k++;
                                    }
                            }
                            link1[t] = t1;
                            if (tgt >= 0) ok &= uf_unite(lab, u, tgt);
                        }
                    } else
                    for_overlap([&](int u) {
                        // the neighbour list four entries at a time: four
                        // independent loads, then four flag loads
                        int k = 0, tgt = -1;
                        const int e1 = brow[u + 1];
                        for (int a = brow[u]; a < e1 && tgt < 0; a += 4) {
                            int v[4];
                            bool on[4];
#pragma unroll
                            for (int j = 0; j < 4; j++) v[j] = a + j < e1 ? (int)(badj[a + j] >> 8) : u;
#pragma unroll
                            for (int j = 0; j < 4; j++) on[j] = a + j < e1 && d[v[j]];
#pragma unroll
                            for (int j = 0; j < 4; j++)
                                if (on[j] && tgt < 0 && k++ == round) tgt = v[j];
                        }
                        if (tgt >= 0) ok &= uf_unite(lab, u, tgt);
                    });
                    team.sync();
                    if (threadIdx.x == 0) P.subtick(round == 0 ? PROF_UF_LINK0 : PROF_UF_LINK1);
                    if (round == 0) {
                        // (after the last round the vote's and phase 3's
                        // finds halve the paths they walk)
                        if (glink) {
                            // four list entries loaded side by side
                            for (int t = team.tr; t < llen; t += 4 * team.ts) {
                                int u[4];
#pragma unroll
                                for (int k = 0; k < 4; k++) {
                                    const int tk = t + k * team.ts;
                                    u[k] = tk < llen ? lst[l0 + tk] : -1;
                                }
#pragma unroll
                                for (int k = 0; k < 4; k++) {
                                    if (u[k] < 0) continue;
                                    const int r = uf_find(vl, u[k]);
                                    if (r < 0) ok = false;
                                    else vl[u[k]] = r;
                                }
                            }
                        } else
                        for_overlap([&](int u) {
                            const int r = uf_find(vl, u);
                            if (r < 0) ok = false;
                            else vl[u] = r;
                        });
                        team.sync();
                        if (threadIdx.x == 0) P.subtick(PROF_UF_COMPRESS);
                    }
                }
                int L = -1;
                if (BLOCK || team.tr < 32) {
                    // vote over 32 sampled overlap sites: a block team samples
                    // its overlap list, every warp the same 32 entries, so
                    // that each warp knows the winner without a barrier (the
                    // roots do not change until the next union); in a warp
                    // team each lane takes the first overlap site in a
                    // 32-byte window of the flags (eight independent word
                    // loads; the flags start on 16 bytes, bytes from n on are
                    // masked)
                    int cand = -1;
                    if (BLOCK) {
                        cand = uf_find(vl, lst[l0 + (int)(((long long)(threadIdx.x & 31) * llen) >> 5)]);
                    } else {
                        const int w0 = (int)(((long long)team.tr * n) >> 7);
                        uint32_t fw[8];
#pragma unroll
                        for (int j = 0; j < 8; j++)
                            fw[j] = 4 * (w0 + j) < n ? reinterpret_cast<const uint32_t*>(d)[w0 + j] : 0u;
                        for (int j = 0; j < 8 && cand < 0; j++)
                            for (int b = 0; b < 4; b++) {
                                const int i = 4 * (w0 + j) + b;
                                if (i < n && ((fw[j] >> (8 * b)) & 0xffu)) { cand = uf_find(vl, i); break; }
                            }
                    }
                    const unsigned grp = __match_any_sync(0xffffffffu, cand);
                    int votes = cand >= 0 ? __popc(grp) : 0, best = cand;
                    for (int o = 16; o > 0; o >>= 1) {
                        const int ov = __shfl_xor_sync(0xffffffffu, votes, o);
                        const int oc = __shfl_xor_sync(0xffffffffu, best, o);
                        if (ov > votes || (ov == votes && oc < best)) { votes = ov; best = oc; }
                    }
                    if (BLOCK) L = best;
                    else if (team.tr == 0) team.ctl[0] = best;
                }
                if (!BLOCK) {
                    team.sync();
                    L = *(volatile int*)team.ctl;
                }
                if (threadIdx.x == 0) P.subtick(PROF_UF_VOTE);
                for_overlap([&](int u) {
                    if (uf_find(vl, u) == L) return;
                    if (BLOCK) {
                        // S never outgrows the free part of lst: |S| <= llen <= n - llen
                        const int pos = atomicAdd(team.ctl + 4, 1);
                        if (pos < llen) lst[sbase + pos] = u;
                        return;
                    }
                    const int e1 = brow[u + 1];
#pragma unroll 4
                    for (int a = brow[u]; a < e1; a++) {
                        const int v = (int)(badj[a] >> 8);
                        if (d[v]) ok &= uf_unite(lab, u, v);
                    }
                });
                team.sync();
                if (threadIdx.x == 0) P.subtick(PROF_UF_OUTSIDE);
                if (BLOCK) {
                    // the edges of S: one warp per site and one lane per
                    // neighbour (the unions of a site side by side) when
                    // that takes fewer rounds than one thread per site
                    const int ns0 = min(*(volatile int*)(team.ctl + 4), llen);
                    const int nw = team.ts >> 5;
                    const bool by_warp = (ns0 + nw - 1) / nw < (D.nnz + n - 1) / n;
                    const int t0 = by_warp ? team.tr >> 5 : team.tr, dt = by_warp ? nw : team.ts;
                    const int a0 = by_warp ? team.tr & 31 : 0, da = by_warp ? 32 : 1;
                    for (int t = t0; t < ns0; t += dt) {
                        const int u = lst[sbase + t];
                        const int e1 = brow[u + 1];
                        for (int a = brow[u] + a0; a < e1; a += da) {
                            const int v = (int)(badj[a] >> 8);
                            if (d[v]) ok &= uf_unite(lab, u, v);
                        }
                    }
                    team.sync();
                    if (threadIdx.x == 0) P.subtick(PROF_UF_SUNION);
                }
                if (BLOCK) {
                    // sites in L's component at their phase-3 check stay in it:
                    // every site outside the final component of L is in S
                    ns = min(*(volatile int*)(team.ctl + 4), llen);
                    const int rL = uf_find(vl, L), rs = uf_find(vl, seed);
                    long long c = 0;   // |S \ comp(L)| when the seed is in comp(L), else |C|
                    for (int t = team.tr; t < ns; t += team.ts) {
                        const int r = uf_find(vl, lst[sbase + t]);
                        c += (rs == rL) ? (r != rL) : (r == rs);
                    }
                    unsigned long long m1 = ~0ull, m2 = ~0ull;
                    long long none = 0;
                    team.reduce(c, m1, m2, none);
                    // every thread has read the list counters: reset them
                    // for the next pair (a barrier of this pair's flip or
                    // energy reduction comes before its next use)
                    if (team.tr == 0) { team.ctl[2] = 0; team.ctl[3] = 0; team.ctl[4] = 0; }
                    csize = (rs == rL) ? cnt - c : c;
                    const bool sw = !exact && csize * 2 > cnt;
                    fast = (rs == rL) ? sw : !sw;   // the flipped set lies in S
                    fast_root = rs == rL ? rL : rs;
                    fast_eq = rs != rL;
                    if (threadIdx.x == 0) P.subtick(PROF_UF_SIZE);
                }
            } else {
                // minimum-label propagation with root hooking and pointer jumping
                // (Shiloach-Vishkin style); labels only decrease and always name
                // a site of the same component
                bool conv = false;
                for (int round = 0; round < 512 && !conv; round++) {
                    int changed = 0;
                    for (int u = team.tr; u < n; u += team.ts) {
                        if (!d[u]) continue;
                        const int lu = vl[u];
                        int best = lu;
                        const int e1 = brow[u + 1];
#pragma unroll 4
                        for (int a = brow[u]; a < e1; a++) {
                            const int v = (int)(badj[a] >> 8);
                            const int lv = vl[v];
                            if (d[v]) best = min(best, lv);
                        }
                        if (best < lu) {
                            atomicMin(lab + lu, best);
                            atomicMin(lab + u, best);
                            changed = 1;
                        }
                    }
                    conv = !(BLOCK ? (__syncthreads_or(changed) != 0) : (__any_sync(0xffffffffu, changed) != 0));
                    if (!BLOCK) __syncwarp();
                    for (int u = team.tr; u < n; u += team.ts) {
                        if (!d[u]) continue;
                        int l = vl[u];
                        for (int g = 0; g < n; g++) {
                            const int ll = vl[l];
                            if (ll >= l) break;
                            l = ll;
                        }
                        vl[u] = l;
                    }
                    team.sync();
                }
                ok = conv;
            }
            if (!ok) dev_fail(A.status, A.abort_flag, DEV_UF_LIMIT, where_err + 3, q, algo);
            if (threadIdx.x == 0) P.subtick(PROF_ICM_UNION);
            const int root = (algo == ENGINE_ICM_UNION_FIND) ? uf_find(vl, seed) : vl[seed];
            if (BLOCK && algo == ENGINE_ICM_UNION_FIND) {
                // csize is known.  When the flipped set is not in S it is the
                // rest of the overlap: mark the selected part of S (d = 3),
                // and the flipped set is every overlap site not marked
                if (!fast) {
                    for (int t = team.tr; t < ns; t += team.ts) {
                        const int u = lst[sbase + t];
                        if ((uf_find(vl, u) == fast_root) == fast_eq) d[u] = 3;
                    }
                    team.sync();
                }
            } else {
                // mark the cluster C (d = 2) and count it
                for_overlap([&](int u) {
                    const int lu = (algo == ENGINE_ICM_UNION_FIND) ? uf_find(vl, u) : vl[u];
                    if (lu != root) return;
                    d[u] = 2;
                    csize++;
                });
                unsigned long long m1 = ~0ull, m2 = ~0ull;
                long long none = 0;
                team.reduce(csize, m1, m2, none);
            }
        }
        // (A, B) -> (A flipped on C, B flipped on C) is the same pair of
        // states as (B flipped on D\C, A flipped on D\C): flip the smaller of
        // C and D\C.  With D\C the pair's two chains hold each other's
        // result at this temperature -- the ICM move followed by an exchange
        // of the two chains' configurations at one temperature, which leaves
        // the joint distribution of the (independent, identical) chains
        // invariant.  Replay keeps the reference's flips.
        swapped = (!exact && csize * 2 > cnt) ? 1 : 0;
        const uint8_t fmark = swapped ? 1 : 2;
        const long long fsize = swapped ? cnt - csize : csize;
        // membership of an overlap site in the flipped set
        const bool rest = BLOCK && algo == ENGINE_ICM_UNION_FIND && !fast;
        auto in_flip = [&](int u) { return rest ? d[u] != 3 : d[u] == fmark; };
        // one pass over a flipped site: flip it and push its field change to
        // its neighbours; the energy changes by the edges leaving the flipped
        // set F.  F is a union of overlap components, so a neighbour outside
        // F is outside the overlap (equal in A and B) and keeps its spin.
        // (by_warp: the lanes of a warp share the site, read its spins
        // before lane 0 flips them and take every 32nd edge)
        auto flip_push = [&](int u, bool by_warp) {
            const int hu = has_h ? bh[u] : 0;
            const int lane = by_warp ? (threadIdx.x & 31) : 0;
            int sa = 0, sb = 0;   // spins before the flip
            if (locA) sa = sA[u];
            if (locB) sb = sB[u];
            if (by_warp) __syncwarp();
            if (lane == 0) {
                if (locA) { sA[u] = (int8_t)-sa; dEa -= 2 * sa * hu; }
                if (locB) { sB[u] = (int8_t)-sb; dEb -= 2 * sb * hu; }
            }
            const int e1 = brow[u + 1], da = by_warp ? 32 : 1;
#pragma unroll 4
            for (int a = brow[u] + lane; a < e1; a += da) {
                const uint32_t e = badj[a];
                const int v = (int)(e >> 8);
                const int J = (int)(int8_t)(e & 0xffu);
                if (fA) atomicAdd(fA + v, J * (-2 * sa));
                if (fB) atomicAdd(fB + v, J * (-2 * sb));
                if (!d[v]) {
                    const int sv = locA ? sA[v] : sB[v];
                    if (locA) dEa -= 2 * J * sa * sv;
                    if (locB) dEb -= 2 * J * sb * sv;
                }
            }
        };
        if (fast) {
            // one warp per site when that takes fewer rounds (as for the
            // unions of S); the membership test is the same in every lane
            const int nw = team.ts >> 5;
            const bool by_warp = BLOCK && (ns + nw - 1) / nw < (D.nnz + n - 1) / n;
            const int t0 = by_warp ? team.tr >> 5 : team.tr, dt = by_warp ? nw : team.ts;
            for (int t = t0; t < ns; t += dt) {
                const int u = lst[sbase + t];
                if ((uf_find((volatile int*)X.queue, u) == fast_root) == fast_eq) flip_push(u, by_warp);
            }
        } else if (BLOCK && fsize * 4 > (long long)n) {
            // a large cluster: flip, then fields and energies from scratch
            // (gathers, no atomics; the cost does not grow with the cluster)
            for_overlap([&](int u) {
                if (!in_flip(u)) return;
                if (locA) sA[u] = (int8_t)-sA[u];
                if (locB) sB[u] = (int8_t)-sB[u];
            });
            team.sync();
            long long eA = 0, eB = 0;
            for (int i = team.tr; i < n; i += team.ts) {
                int fa = 0, fb = 0;
                const int e1 = brow[i + 1];
#pragma unroll 4
                for (int a = brow[i]; a < e1; a++) {
                    const uint32_t e = badj[a];
                    const int v = (int)(e >> 8);
                    const int J = (int)(int8_t)(e & 0xffu);
                    if (locA) fa += J * sA[v];
                    if (locB) fb += J * sB[v];
                }
                const int h2 = has_h ? 2 * bh[i] : 0;
                if (locA) { if (fA) fA[i] = fa; eA += (long long)sA[i] * (h2 + fa); }
                if (locB) { if (fB) fB[i] = fb; eB += (long long)sB[i] * (h2 + fb); }
            }
            team.sum2(eA, eB);
            if (team.tr == 0) {
                if (locA) B.E[rA] = eA / 2;
                if (locB) B.E[rB] = eB / 2;
            }
            absolute = true;
        } else {
            // a small flipped set, flipped and pushed in one pass
            for_overlap([&](int u) {
                if (in_flip(u)) flip_push(u, false);
            });
        }
        team.sync();
    }
    if (!absolute && (gflip || cnt > 0)) {
        team.sum2(dEa, dEb);
        if (team.tr == 0) {
            if (locA) B.E[rA] += dEa;
            if (locB && cnt > 0) B.E[rB] += dEb;
        }
    }
    if (!(BLOCK && algo == ENGINE_ICM_UNION_FIND && cnt > 0)) {
        // (a block team's union-find reset the list counters after its size
        // reduction and passed a barrier since)
        if (BLOCK && team.tr == 0) {
            team.ctl[2] = 0;   // the list counters, for the next pair
            team.ctl[3] = 0;
            team.ctl[4] = 0;
        }
        team.sync();
    }
    if (threadIdx.x == 0) {
        P.subtick(PROF_ICM_FLIP);
        if (P.on && cnt > 0) P.c[PROF_ICM_COUNT]++;
    }
    return swapped;
}

// Local field of site i gathered from the neighbours' spins (field_gather
// mode, where fields are not stored): f_i = sum_j J_ij s_j.
__device__ __forceinline__ int gather_field(const int32_t* row, const uint32_t* adj, const int8_t* sp, int i) {
    int f = 0;
    for_each_neighbour(row, adj, i, [&](uint32_t e) { f += (int)(int8_t)(e & 0xffu) * sp[e >> 8]; });
    return f;
}

// --------------------------------------------------------------- sweeps
// A warp pushes the field changes of at most this many accepted sites one
// site at a time (a lane per neighbour); with more, each lane pushes its own
// (on C2, 4 to 8 measured best: 26.5 us per PT step against 27.6 with every
// lane pushing its own).
constexpr int kCoopPushSites = 4;
// With fields gathered and several replicas in a block, a thread visits one
// site of each of at most this many replicas per neighbour-list read.
constexpr int kGatherReps = 4;

// Colour-class Metropolis sweep of the block's replicas (production).
// dE_i = -2 s_i (h_i + f_i); accepted with probability min(1, exp(-beta dE))
// (src/replica.cc:31-38); an accepted flip pushes J_ij * (-2 s_i) into each
// neighbour's field (the integer form of src/problem.cc:164-181).  With one
// replica per block (ONE) every thread keeps its energy change and flip
// count in registers until a phase boundary; with several, warps aggregate
// per replica before touching shared memory.
template <bool ONE, bool COOP>
__device__ void colored_sweep(const EngineArgs& A, const BlockCtx& B, unsigned long long sweep_idx,
                              int32_t* s_col, const uint32_t* s_thr, int* s_dEp, unsigned* s_flp,
                              unsigned long long* s_flips, long long* s_bestE, int* s_improved,
                              int* s_misc, bool best_per_phase) {
    const InstanceDesc& D = B.D;
    const int T = blockDim.x, tid = threadIdx.x, lane = tid & 31;
    const int npad = D.n_pad, rpc = ONE ? 1 : D.rpc;
    const int32_t* row = B.row;
    const uint32_t* adj = B.adj;
    const int kmax = D.kmax;
    ThreadRng12 rng;
    // counter: (rank in the group, thread), sweep, instance id in the high
    // half of the call word (a thread makes far fewer than 2^16 calls)
    rng.start(stream_key(A.seed, STREAM_SWEEP), (uint32_t)(B.rank * T + tid), sweep_idx, (uint32_t)D.inst_id << 16);
    int acc_de = 0;
    unsigned acc_fl = 0;
    // several replicas in the block, fields gathered
    const bool gm = !ONE && B.field == nullptr && rpc <= kGatherReps;
    // the one-replica sweep's pointers and flags, read once from the
    // block's shared context (the compiler may not keep them across the
    // stores of a colour class)
    int8_t* const sp1 = B.spin;
    int32_t* const fd1 = B.field;
    const int32_t* const h1 = D.has_h ? B.h : nullptr;
    const uint32_t* const thr1 = ONE ? s_thr + B.tb[0] : s_thr;
    const int ncolors = D.ncolors;
    for (int c = 0; c < ncolors; c++) {
        const int c0 = s_col[c];
        const int Sc = s_col[c + 1] - c0;
        if (ONE && COOP && fd1 != nullptr) {
            // each thread decides its own site (the same site and random
            // draws as one site per thread).  A warp with few accepted sites
            // (the cold replicas) pushes their field changes one site at a
            // time with a lane per neighbour, so that no lane walks a long
            // neighbour list alone; a warp with many (the hot replicas)
            // lets every lane push its own site's changes, side by side
            int8_t* const sp = sp1;
            int32_t* const fd = fd1;
            const uint32_t* const thr_row = thr1;
            for (int base = c0 + (tid & ~31); base < c0 + Sc; base += T) {
                const int i = base + lane;
                bool acc = false;
                int s = 0, e0 = 0, e1 = 0;
                if (i < c0 + Sc) {
                    s = sp[i];
                    const int f = fd[i] + (h1 != nullptr ? h1[i] : 0);
                    const int de = -2 * s * f;
                    acc = de <= 0;
                    if (!acc) {
                        const uint32_t thr = thr_row[min(de >> 1, kmax)];
                        acc = (rng.next_one() < thr) || (thr == 0xFFFFFFFFu);
                    }
                    if (acc) {
                        sp[i] = (int8_t)-s;
                        acc_de += de;
                        acc_fl++;
                        e0 = row[i];
                        e1 = row[i + 1];
                    }
                }
                unsigned m = __ballot_sync(0xffffffffu, acc);
                if (__popc(m) > kCoopPushSites) {
                    if (acc) {
                        const int dl = -2 * s;
                        for_each_neighbour(row, adj, i,
                                           [&](uint32_t e) { atomicAdd(fd + (e >> 8), (int)(int8_t)(e & 0xffu) * dl); });
                    }
                    m = 0;
                }
                while (m) {
                    const int src = __ffs(m) - 1;
                    m &= m - 1;
                    const int a0 = __shfl_sync(0xffffffffu, e0, src), a1 = __shfl_sync(0xffffffffu, e1, src);
                    const int dl = -2 * __shfl_sync(0xffffffffu, s, src);
                    for (int a = a0 + lane; a < a1; a += 32) {
                        const uint32_t e = adj[a];
                        atomicAdd(fd + (e >> 8), (int)(int8_t)(e & 0xffu) * dl);
                    }
                }
            }
        } else if (ONE) {
            int8_t* sp = B.spin;
            int32_t* fd = B.field;   // null in field_gather mode
            const uint32_t* thr_row = s_thr + B.tb[0];
            for (int i = c0 + tid; i < c0 + Sc; i += T) {
                const int s = sp[i];
                const int f = (fd ? fd[i] : gather_field(row, adj, sp, i)) + (D.has_h ? B.h[i] : 0);
                const int de = -2 * s * f;
                bool acc = de <= 0;
                if (!acc) {
                    const uint32_t thr = thr_row[min(de >> 1, kmax)];
                    acc = (rng.next() < thr) || (thr == 0xFFFFFFFFu);
                }
                if (acc) {
                    sp[i] = (int8_t)-s;
                    acc_de += de;
                    acc_fl++;
                    if (fd) {
                        const int dl = -2 * s;
                        for_each_neighbour(row, adj, i,
                                           [&](uint32_t e) { atomicAdd(fd + (e >> 8), (int)(int8_t)(e & 0xffu) * dl); });
                    }
                }
            }
        } else if (gm) {
            // a thread visits site i of each of the block's replicas: the
            // neighbour list is read once for all of them (sites of one
            // colour class share no edge, so the gathered spins are settled)
            int g_de[kGatherReps];
            unsigned g_fl[kGatherReps];
#pragma unroll
            for (int j = 0; j < kGatherReps; j++) {
                g_de[j] = 0;
                g_fl[j] = 0;
            }
            for (int i = c0 + tid; i < c0 + Sc; i += T) {
                int f[kGatherReps];
#pragma unroll
                for (int j = 0; j < kGatherReps; j++) f[j] = 0;
                // the neighbour list 16 bytes at a time, one load in flight
                // (four spin loads per entry keep the thread busy)
                auto scan = [&](auto&& visit) {
                    int a = row[i];
                    const int a1 = row[i + 1];
                    if ((reinterpret_cast<uintptr_t>(adj) & 15u) == 0) {
                        for (; a < a1 && (a & 3); a++) visit(adj[a]);
#pragma unroll 1
                        for (; a + 4 <= a1; a += 4) {
                            const uint4 q = *reinterpret_cast<const uint4*>(adj + a);
                            visit(q.x);
                            visit(q.y);
                            visit(q.z);
                            visit(q.w);
                        }
                    }
                    for (; a < a1; a++) visit(adj[a]);
                };
                scan([&](uint32_t e) {
                    const int w = (int)(int8_t)(e & 0xffu);
                    const int8_t* sn = B.spin + (e >> 8);
#pragma unroll
                    for (int j = 0; j < kGatherReps; j++)
                        if (j < rpc) f[j] += w * sn[j * npad];
                });
                const int hi = D.has_h ? B.h[i] : 0;
#pragma unroll
                for (int j = 0; j < kGatherReps; j++) {
                    if (j < rpc) {
                        int8_t* sp = B.spin + j * npad;
                        const int s = sp[i];
                        const int de = -2 * s * (f[j] + hi);
                        bool acc = de <= 0;
                        if (!acc) {
                            const uint32_t thr = s_thr[B.tb[j] + min(de >> 1, kmax)];
                            acc = (rng.next() < thr) || (thr == 0xFFFFFFFFu);
                        }
                        if (acc) {
                            sp[i] = (int8_t)-s;
                            g_de[j] += de;
                            g_fl[j]++;
                        }
                    }
                }
            }
#pragma unroll
            for (int j = 0; j < kGatherReps; j++) {
                if (j < rpc) {
                    int v = g_de[j];
                    unsigned f = g_fl[j];
                    for (int o = 16; o > 0; o >>= 1) {
                        v += __shfl_xor_sync(0xffffffffu, v, o);
                        f += __shfl_xor_sync(0xffffffffu, f, o);
                    }
                    if (lane == 0 && (v != 0 || f != 0)) {
                        atomicAdd(s_dEp + j, v);
                        atomicAdd(s_flp + j, f);
                    }
                }
            }
        } else {
            const int items = rpc * Sc;
            const int items_w = (items + 31) & ~31;   // whole warps iterate together
            for (int it = tid; it < items_w; it += T) {
                int j = -1, de = 0;
                bool acc = false;
                if (it < items) {
                    j = it / Sc;
                    const int i = c0 + (it - j * Sc);
                    int8_t* sp = B.spin + j * npad;
                    int32_t* fd = B.field ? B.field + j * npad : nullptr;
                    const int s = sp[i];
                    const int f = (fd ? fd[i] : gather_field(row, adj, sp, i)) + (D.has_h ? B.h[i] : 0);
                    de = -2 * s * f;
                    acc = de <= 0;
                    if (!acc) {
                        const uint32_t thr = s_thr[B.tb[j] + min(de >> 1, kmax)];
                        acc = (rng.next() < thr) || (thr == 0xFFFFFFFFu);
                    }
                    if (acc) {
                        sp[i] = (int8_t)-s;
                        if (fd) {
                            const int dl = -2 * s;
                            for_each_neighbour(row, adj, i, [&](uint32_t e) {
                                atomicAdd(fd + (e >> 8), (int)(int8_t)(e & 0xffu) * dl);
                            });
                        }
                    }
                }
                // one shared-memory update per replica per warp instead of per flip
                const int key = acc ? j : -1;
                const unsigned grp = __match_any_sync(0xffffffffu, key);
                if (acc) {
                    const int sde = __reduce_add_sync(grp, de);
                    if (lane == __ffs(grp) - 1) {
                        atomicAdd(s_dEp + j, sde);
                        atomicAdd(s_flp + j, (unsigned)__popc(grp));
                    }
                }
            }
        }
        const bool track = best_per_phase || c + 1 == D.ncolors;
        if (ONE && track) {
            int v = acc_de;
            unsigned f = acc_fl;
            for (int o = 16; o > 0; o >>= 1) {
                v += __shfl_xor_sync(0xffffffffu, v, o);
                f += __shfl_xor_sync(0xffffffffu, f, o);
            }
            if (lane == 0 && (v != 0 || f != 0)) {
                atomicAdd(s_dEp, v);
                atomicAdd(s_flp, f);
            }
            acc_de = 0;
            acc_fl = 0;
        }
        __syncthreads();
        if (!track) continue;
        // phase boundary: fold the phase's energy change, track the best state
        for (int jj = tid; jj < rpc; jj += T) {
            const int r = B.r0 + jj;
            const long long E = B.E[r] + s_dEp[jj];
            B.E[r] = E;
            s_dEp[jj] = 0;
            s_flips[jj] += s_flp[jj];
            s_flp[jj] = 0;
            const bool imp = E < s_bestE[jj];
            s_improved[jj] = imp;
            if (imp) {
                s_bestE[jj] = E;
                A.best_sweep[D.rep_off + r] = sweep_idx;
                atomicAdd(s_misc + 1, 1);
            }
        }
        __syncthreads();
        if (s_misc[1] > 0) {
            for (int idx = tid; idx < rpc * npad; idx += T) {
                const int j = ONE ? 0 : idx / npad;
                if (s_improved[j]) A.best_state[D.spin_off + (long long)B.r0 * npad + idx] = B.spin[idx];
            }
            __syncthreads();
            if (tid == 0) s_misc[1] = 0;
            __syncthreads();
        }
    }
}

// Sequential sweep in the reference's site order (replay).  One warp per
// replica: lane 0 makes each decision exactly as src/replica.cc:31-38 does
// (dE <= 0, else u < exp(-beta*dE) with a recorded u), the warp applies the
// field update and copies a new best state (src/replica.cc:18-29).
__device__ void replay_sweep(const EngineArgs& A, const BlockCtx& B, int ls, int sw,
                             unsigned long long sweep_idx, const double* s_ptab,
                             unsigned long long* s_flips, long long* s_bestE) {
    const InstanceDesc& D = B.D;
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5, nw = blockDim.x >> 5;
    const int n = D.n, npad = D.n_pad, kst = D.kmax + 1;
    for (int j = warp; j < D.rpc; j += nw) {
        const int r = B.r0 + j;
        int8_t* sp = B.spin + j * npad;
        int32_t* fd = B.field + j * npad;
        const long long oi = ((long long)ls * A.sweeps + sw) * D.R + r;
        unsigned long long pos = A.replay.sweep_offsets[oi];
        const unsigned long long end = A.replay.sweep_offsets[oi + 1];
        const int pbase = (int)(B.rslot[j] % (uint32_t)D.nt) * kst;
        long long E = B.E[r];
        long long bestE = s_bestE[j];
        unsigned long long flips = 0;
        bool bad = false;
        for (int o = 0; o < n; o++) {
            const int i = A.perm[D.perm_off + o];
            int acc = 0, s = 0, de = 0;
            if (lane == 0) {
                s = sp[i];
                const int f = fd[i] + (D.has_h ? B.h[i] : 0);
                de = -2 * s * f;
                if (de <= 0) {
                    acc = 1;
                } else {
                    double u = 1.0;
                    if (pos < end && pos < A.replay.n_uniforms) u = A.replay.uniforms[pos];
                    else bad = true;
                    pos++;
                    acc = u < s_ptab[pbase + min(de >> 1, D.kmax)];
                }
            }
            acc = __shfl_sync(0xffffffffu, acc, 0);
            if (!acc) continue;
            s = __shfl_sync(0xffffffffu, s, 0);
            de = __shfl_sync(0xffffffffu, de, 0);
            if (lane == 0) sp[i] = (int8_t)-s;
            const int e0 = B.row[i], e1 = B.row[i + 1];
            for (int a = e0 + lane; a < e1; a += 32) {
                const uint32_t e = B.adj[a];
                atomicAdd(fd + (e >> 8), (int)(int8_t)(e & 0xffu) * (-2 * s));
            }
            E += de;
            flips++;
            __syncwarp();
            if (E < bestE) {
                bestE = E;
                for (int x = lane; x < npad; x += 32) A.best_state[D.spin_off + (long long)r * npad + x] = sp[x];
                if (lane == 0) A.best_sweep[D.rep_off + r] = sweep_idx;
            }
            __syncwarp();
        }
        if (lane == 0) {
            if (bad || pos != end) dev_fail(A.status, A.abort_flag, DEV_REPLAY_MISMATCH, 10, oi, (long long)(end - pos));
            B.E[r] = E;
            s_bestE[j] = bestE;
            s_flips[j] += flips;
        }
        __syncwarp();
    }
}

// ------------------------------------------------------------- exchange
// Production exchange with the reference's attempt order
// (src/replica_exchange.cc:5-100): a shuffled order of the nt-1 adjacent
// pairs is walked by one cursor shared by all chains (attempt a goes to chain
// a % chains); the order is reshuffled whenever the cursor wraps.  Attempt
// on pair k accepts iff dBeta*dE > 0 or log u < dBeta*dE, and swaps the
// slot->replica entries.  Within one pass over the order each pair appears
// once, so an attempt depends only on earlier attempts on the neighbouring
// pairs of its chain: attempts are grouped into dependency levels and each
// level runs in parallel, with exactly the sequential semantics.
__device__ void exchange_reference_order(const EngineArgs& A, const BlockCtx& B, unsigned long long step,
                                         uint32_t* s_order, const double* s_dbeta, unsigned* s_att,
                                         unsigned* s_succ, float* s_xlogu, uint32_t* s_xrand,
                                         int* s_lvl, uint32_t* s_tmp, int* s_misc, Prof& P) {
    if (threadIdx.x == 0) P.subtick(PROF_X_SHUFFLE);
    const InstanceDesc& D = B.D;
    const int tid = threadIdx.x, T = blockDim.x;
    const int nt = D.nt, C = D.chains, m = nt - 1;
    if (m <= 0) return;
    const int total = C * m;
    // pre-draw: total log-uniforms and total shuffle keys
    const uint2 key = stream_key(A.seed, STREAM_EXCHANGE);
    const int ndraw = 2 * total;
    for (int call = tid; call * 4 < ndraw; call += T) {
        const uint4 r = philox4x32_10(make_uint4((uint32_t)call, (uint32_t)D.inst_id, (uint32_t)step,
                                                 (uint32_t)(step >> 32)), key);
        const uint32_t v[4] = {r.x, r.y, r.z, r.w};
#pragma unroll
        for (int q = 0; q < 4; q++) {
            const int dix = call * 4 + q;
            if (dix < total) s_xlogu[dix] = __logf(u01_open0(v[q]));
            else if (dix < ndraw) s_xrand[dix - total] = v[q];
        }
    }
    __syncthreads();
    if (threadIdx.x == 0) P.subtick(PROF_X_DRAW);
    // one warp walks the rounds; the rest of the block waits at the end
    if (tid < 32) {
        const int lane = tid;
        for (int round = 0; round < C; round++) {
            // level of attempt i = 1 + max level of earlier attempts on the
            // neighbouring pairs of the same chain
            for (int i = lane; i < m; i += 32) {
                s_lvl[i] = 1;
                s_tmp[s_order[i]] = (uint32_t)i;   // position of each pair in this pass
            }
            __syncwarp();
            for (int iter = 0; iter <= m; iter++) {
                int changed = 0;
                for (int i = lane; i < m; i += 32) {
                    const int kb = (int)s_order[i];
                    const int c = (round * m + i) % C;
                    int lv = 1;
                    if (kb > 0) {
                        const int jn = (int)s_tmp[kb - 1];
                        if (jn < i && (round * m + jn) % C == c) lv = max(lv, ((volatile int*)s_lvl)[jn] + 1);
                    }
                    if (kb + 1 < m) {
                        const int jn = (int)s_tmp[kb + 1];
                        if (jn < i && (round * m + jn) % C == c) lv = max(lv, ((volatile int*)s_lvl)[jn] + 1);
                    }
                    if (lv != s_lvl[i]) { s_lvl[i] = lv; changed = 1; }
                }
                const bool again = __any_sync(0xffffffffu, changed);
                __syncwarp();
                if (!again) break;
            }
            int maxl = 0;
            for (int i = lane; i < m; i += 32) maxl = max(maxl, s_lvl[i]);
            const int L = __reduce_max_sync(0xffffffffu, maxl);
            if (lane == 0) P.subtick(PROF_X_LEVELS);
            for (int lv = 1; lv <= L; lv++) {
                for (int i = lane; i < m; i += 32) {
                    if (s_lvl[i] != lv) continue;
                    const int kb = (int)s_order[i];
                    const int a = round * m + i;
                    const int c = a % C;
                    const int k = c * nt + kb;
                    const uint32_t r1 = B.slot[k], r2 = B.slot[k + 1];
                    const double x = s_dbeta[kb] * (double)(B.E[r1] - B.E[r2]);
                    s_att[k]++;
                    if (x > 0.0 || (double)s_xlogu[a] < x) {
                        s_succ[k]++;
                        B.slot[k] = r2;
                        B.slot[k + 1] = r1;
                    }
                }
                __syncwarp();
            }
            if (lane == 0) P.subtick(PROF_X_APPLY);
            // reshuffle: rank the pairs by fresh random keys (ties by position)
            const uint32_t* keys = s_xrand + round * m;
            for (int i = lane; i < m; i += 32) {
                const uint32_t ki = keys[i];
                int rank = 0;
                for (int j = 0; j < m; j++) {
                    const uint32_t kj = keys[j];
                    rank += (kj < ki) || (kj == ki && j < i);
                }
                s_tmp[rank] = s_order[i];
            }
            __syncwarp();
            for (int i = lane; i < m; i += 32) s_order[i] = s_tmp[i];
            __syncwarp();
            if (lane == 0) P.subtick(PROF_X_SHUFFLE);
        }
    }
    __syncthreads();
    (void)s_misc;
}

// Deterministic even/odd exchange: per chain, all even pairs, then all odd
// pairs, each set in parallel (nt-1 attempts per chain per step).
__device__ void exchange_even_odd(const EngineArgs& A, const BlockCtx& B, unsigned long long step,
                                  const double* s_dbeta, unsigned* s_att, unsigned* s_succ) {
    const InstanceDesc& D = B.D;
    const int tid = threadIdx.x, T = blockDim.x;
    const int nt = D.nt, C = D.chains, m = nt - 1;
    const uint32_t inst = (uint32_t)D.inst_id;
    uint32_t* const slot = B.slot;
    const long long* const E = B.E;
    const uint2 key = stream_key(A.seed, STREAM_EXCHANGE);
    auto log_u = [&](int k, int par) {
        const uint4 r = philox4x32_10(make_uint4((uint32_t)(k | (par << 30)), inst, (uint32_t)step, (uint32_t)(step >> 32)), key);
        return __logf(u01_open0(r.x));
    };
    auto pair_of = [&](int t, int par, int per_chain, int& kb) {
        const int c = t / per_chain;
        kb = par + 2 * (t - c * per_chain);
        return c * nt + kb;
    };
    // when each pass has at most one pair per thread, both passes' draws
    // are made first, side by side (they do not depend on the energies)
    const int per0 = (m + 1) / 2, per1 = m / 2;
    const bool one = C * per0 <= T;
    float lu0 = 0.f, lu1 = 0.f;
    if (one) {
        int kb;
        if (tid < C * per0) lu0 = log_u(pair_of(tid, 0, per0, kb), 0);
        if (tid < C * per1) lu1 = log_u(pair_of(tid, 1, per1, kb), 1);
    }
    for (int par = 0; par < 2; par++) {
        const int per_chain = par ? per1 : per0;   // pairs kb = par, par+2, ...
        const int total = C * per_chain;
        for (int t = tid; t < total; t += T) {
            int kb;
            const int k = pair_of(t, par, per_chain, kb);
            const float lu = one ? (par ? lu1 : lu0) : log_u(k, par);
            const uint32_t r1 = slot[k], r2 = slot[k + 1];
            const double x = s_dbeta[kb] * (double)(E[r1] - E[r2]);
            s_att[k]++;
            if (x > 0.0 || (double)lu < x) {
                s_succ[k]++;
                slot[k] = r2;
                slot[k + 1] = r1;
            }
        }
        __syncthreads();
    }
}

// Replayed exchange: the recorded pair sequence and log-uniforms, applied
// sequentially in FP64 exactly as src/replica_exchange.cc:20-40 computes.
__device__ void exchange_replay(const EngineArgs& A, const BlockCtx& B, int ls, const double* s_beta,
                                unsigned* s_att, unsigned* s_succ) {
    const InstanceDesc& D = B.D;
    if (threadIdx.x == 0) {
        const int nt = D.nt, per = D.chains * (nt - 1);
        for (int t = 0; t < per; t++) {
            const long long idx = (long long)ls * per + t;
            if (idx >= (long long)A.replay.n_xchg) {
                dev_fail(A.status, A.abort_flag, DEV_REPLAY_MISMATCH, 20, idx, 0);
                break;
            }
            const int k = A.replay.xchg_slot[idx];
            if (k < 0 || k + 1 >= D.R || (k % nt) == nt - 1) {
                dev_fail(A.status, A.abort_flag, DEV_BAD_INDEX, 21, idx, k);
                break;
            }
            const int kb = k % nt;
            const uint32_t r1 = B.slot[k], r2 = B.slot[k + 1];
            const double dB = __dsub_rn(s_beta[kb], s_beta[kb + 1]);
            const double dE = (double)(B.E[r1] - B.E[r2]);
            const double x = __dmul_rn(dB, dE);
            s_att[k]++;
            if (__dmul_rn(dE, dB) > 0.0 || A.replay.xchg_logu[idx] < x) {
                s_succ[k]++;
                B.slot[k] = r2;
                B.slot[k + 1] = r1;
            }
        }
    }
    __syncthreads();
}

// ---------------------------------------------------------------- kernel
// Launch bounds: blocks of several replicas, and narrow block teams (NARROW),
// run at most kNarrowThreads threads, which leaves each thread 120 registers
// instead of the 64 of a 1024-thread bound; replay and wide block teams (one
// replica of a large instance per block) keep 1024.
template <bool REPLAY, bool BLOCKTEAM, bool NARROW>
__global__ void __launch_bounds__((REPLAY || (BLOCKTEAM && !NARROW)) ? 1024 : kNarrowThreads, 1)
    pt_engine_kernel(const EngineArgs A) {
    extern __shared__ __align__(128) uint8_t smem[];
    // the job's context and the profiling counters: one copy per block (per-
    // thread copies of uniform values would live in local memory)
    __shared__ BlockCtx s_B;
    __shared__ long long s_prof[PROF_PHASES];
    const SmemPlan& S = A.sm;
    const int tid = threadIdx.x, T = blockDim.x;
    volatile int* abortf = A.abort_flag;
    uint64_t* mbar = sm_ptr<uint64_t>(smem, S.mbar);
    if (S.stage_adj) {
        if (tid == 0) mbar_init(mbar, 1);
        __syncthreads();
    }
    uint32_t bulk_parity = 0;
    const int job_end = A.sched_off[blockIdx.x + 1];
    for (int job = A.sched_off[blockIdx.x]; job < job_end; job++) {
    const int inst = A.sched[2 * job];
    if (tid == 0) {
        s_B.D = A.desc[inst];
        s_B.rank = A.sched[2 * job + 1];
        s_B.r0 = s_B.rank * s_B.D.rpc;
    }
    __syncthreads();
    BlockCtx& B = s_B;
    const InstanceDesc& D = B.D;
    const int n = D.n, npad = D.n_pad, R = D.R, nt = D.nt, rpc = D.rpc, kst = D.kmax + 1;

    int32_t* s_col = sm_ptr<int32_t>(smem, S.col);
    int32_t* s_h = sm_ptr<int32_t>(smem, S.h);
    // acceptance thresholds: shared memory, or read through L1 (field_gather)
    uint32_t* s_thr_w = sm_ptr<uint32_t>(smem, S.thr);
    const uint32_t* s_thr = S.field_gather ? A.thr + D.thr_off : s_thr_w;
    double* s_ptab = sm_ptr<double>(smem, S.ptab);
    uint32_t* s_order = sm_ptr<uint32_t>(smem, S.order);
    double* s_beta = sm_ptr<double>(smem, S.beta);
    double* s_dbeta = sm_ptr<double>(smem, S.dbeta);
    int* s_dEp = sm_ptr<int>(smem, S.dEp);
    unsigned* s_flp = sm_ptr<unsigned>(smem, S.flp);
    long long* s_bestE = sm_ptr<long long>(smem, S.bestE);
    unsigned long long* s_flips = sm_ptr<unsigned long long>(smem, S.flips);
    int* s_improved = sm_ptr<int>(smem, S.improved);
    unsigned* s_att = sm_ptr<unsigned>(smem, S.att);
    unsigned* s_succ = sm_ptr<unsigned>(smem, S.succ);
    float* s_xlogu = sm_ptr<float>(smem, S.xlogu);
    uint32_t* s_xrand = sm_ptr<uint32_t>(smem, S.xrand);
    int* s_lvl = sm_ptr<int>(smem, S.xlevel);
    uint32_t* s_tmp = sm_ptr<uint32_t>(smem, S.xpos);
    uint8_t* s_icm = ((S.state_global || S.field_gather) && !S.icm_split)
                         ? A.icm_pool + (size_t)blockIdx.x * (size_t)A.icm_pool_stride
                         : smem + S.icm;
    int* s_misc = sm_ptr<int>(smem, S.misc);
    long long* s_mag = sm_ptr<long long>(smem, S.mag);
    long long* s_team_acc = sm_ptr<long long>(smem, S.misc + 64);
    int* s_team_bc = sm_ptr<int>(smem, S.misc + 64 + 8 * 32);   // 2 ints per team

    const int32_t* g_row = A.row + D.row_off;
    const uint32_t* g_adj = A.adj + D.adj_off;

    // ---- stage the adjacency (bulk copies) and load the block's state
    bool staged = S.stage_adj && D.stage;
    if (staged && ((reinterpret_cast<uintptr_t>(g_row) | reinterpret_cast<uintptr_t>(g_adj)) & 15u)) {
        // a bulk copy needs 16-byte aligned sources: record and skip it
        if (tid == 0) dev_fail(A.status, A.abort_flag, DEV_BAD_INDEX, 3, blockIdx.x, inst);
        staged = false;
    }
    if (staged) {
        int32_t* s_row = sm_ptr<int32_t>(smem, S.row);
        uint32_t* s_adj = sm_ptr<uint32_t>(smem, S.adj);
        if (tid == 0) {
            // the previous job's generic-proxy reads of this region are done
            // (block barrier at the end of every job); order them before the
            // bulk copy's writes
            asm volatile("fence.proxy.async.shared::cta;" ::: "memory");
            const uint32_t rb = (uint32_t)(((n + 1) * 4 + 15) & ~15);
            const uint32_t ab = (uint32_t)((D.nnz * 4 + 15) & ~15);
            mbar_expect_tx(mbar, rb + ab);
            bulk_g2s(s_row, g_row, rb, mbar);
            if (ab) bulk_g2s(s_adj, g_adj, ab, mbar);
        }
    }
    if (tid == 0) {
        if (S.state_global) {
            // replicas too large for shared memory work on their master copy
            B.spin = A.spins + D.spin_off + (long long)B.r0 * D.n_pad;
            B.field = A.fields + D.spin_off + (long long)B.r0 * D.n_pad;
        } else {
            B.spin = sm_ptr<int8_t>(smem, S.spin);
            B.field = S.field_gather ? nullptr : sm_ptr<int32_t>(smem, S.field);
        }
        B.slot = sm_ptr<uint32_t>(smem, S.slot);
        B.rslot = sm_ptr<uint32_t>(smem, S.rslot);
        B.tb = sm_ptr<int32_t>(smem, S.rslot) + rpc;
        B.E = sm_ptr<long long>(smem, S.E);
        B.h = D.has_h ? s_h : nullptr;
        B.row = staged ? sm_ptr<int32_t>(smem, S.row) : g_row;
        B.adj = staged ? sm_ptr<uint32_t>(smem, S.adj) : g_adj;
    }
    __syncthreads();
    for (int i = tid; i <= D.ncolors; i += T) s_col[i] = A.col[D.col_off + i];
    if (D.has_h)
        for (int i = tid; i < n; i += T) s_h[i] = A.hpool[D.h_off + i];
    if (!S.state_global) {
        const long long base = D.spin_off + (long long)B.r0 * npad;
        for (int idx = tid; idx < rpc * npad; idx += T) {
            B.spin[idx] = A.spins[base + idx];
            if (B.field) B.field[idx] = A.fields[base + idx];
        }
    }
    for (int r = tid; r < R; r += T) {
        B.slot[r] = A.slot_rep[D.rep_off + r];
        B.E[r] = A.energy[D.rep_off + r];
        s_att[r] = 0;
        s_succ[r] = 0;
    }
    for (int k = tid; k < nt; k += T) {
        s_order[k] = A.xorder[D.rep_off + k];
        s_beta[k] = A.beta[D.beta_off + k];
    }
    for (int k = tid; k < nt * kst; k += T) {
        if (!S.field_gather) s_thr_w[k] = A.thr[D.thr_off + k];
        if (REPLAY) s_ptab[k] = A.ptab[D.ptab_off + k];
    }
    for (int j = tid; j < rpc; j += T) {
        s_bestE[j] = A.best_E[D.rep_off + B.r0 + j];
        s_flips[j] = 0;
        s_dEp[j] = 0;
        s_flp[j] = 0;
        s_improved[j] = 0;
    }
    if (tid < 8) s_misc[tid] = 0;
    // the group barrier's generation (it cannot move before this block arrives)
    unsigned int bar_gen = 0;
    if (tid == 0 && D.group > 1) bar_gen = *(volatile unsigned int*)(A.bar + 2 * inst + 1);
    if (tid == 0) {
        for (int q = 0; q < 3; q++) team_slot_reset(s_team_acc, q);
        s_team_bc[2] = 0;   // the block team's overlap-list and S counters
        s_team_bc[3] = 0;
        s_team_bc[4] = 0;
    }
    __syncthreads();
    for (int k = tid; k + 1 < nt; k += T) s_dbeta[k] = s_beta[k] - s_beta[k + 1];
    for (int s = tid; s < R; s += T) {
        const uint32_t r = B.slot[s];
        if ((int)r >= B.r0 && (int)r < B.r0 + rpc) {
            B.rslot[r - B.r0] = (uint32_t)s;
            B.tb[r - B.r0] = (int)(((uint32_t)s % (uint32_t)nt) * (uint32_t)kst);
        }
    }
    if (staged) {
        if (!mbar_wait_bounded(mbar, bulk_parity, A.wait_limit_ns ? A.wait_limit_ns : kWaitLimitNs) && tid == 0)
            dev_fail(A.status, A.abort_flag, DEV_TMA_TIMEOUT, 2, blockIdx.x, inst);
        bulk_parity ^= 1u;
    }
    __syncthreads();

    const bool icm_on = (A.phase_mask & PHASE_ICM) && D.nc > 0 && D.chains >= 2;
    Prof P;
    P.init((A.prof != nullptr) && tid == 0, s_prof);
    const long long t_start = P.mark;
    const bool best_pp = (A.flags & ENGINE_BEST_PER_PHASE) != 0;
    unsigned long long t_step1 = 0;
    for (int ls = 0; ls < A.nsteps; ls++) {
        if (ls == 1 && tid == 0) t_step1 = globaltimer_ns();
        if (D.group == 1) {
            // (a group of blocks sees an abort in its barrier)
            if (tid == 0) s_misc[3] = *abortf;
            __syncthreads();
            if (s_misc[3]) break;
        }
        const unsigned long long step = A.step0 + (unsigned long long)ls;
        const int parity = (int)(step & 1ull);
        // (profiling) a block holding one replica at an ICM temperature
        const bool cold = P.on && icm_on && rpc == 1 && (nt - 1 - (int)(B.rslot[0] % (uint32_t)nt)) < D.nc;
        const long long t_sw = P.on ? clock64() : 0;
        if (A.phase_mask & PHASE_SWEEP) {
            for (int sw = 0; sw < A.sweeps; sw++) {
                const unsigned long long sweep_idx = step * (unsigned long long)A.sweeps + (unsigned long long)sw;
                if (REPLAY) {
                    replay_sweep(A, B, ls, sw, sweep_idx, s_ptab, s_flips, s_bestE);
                    __syncthreads();
                } else {
                    colored_sweep<BLOCKTEAM, BLOCKTEAM && NARROW>(A, B, sweep_idx, s_col, s_thr, s_dEp, s_flp, s_flips, s_bestE,
                                             s_improved, s_misc, best_pp);
                }
            }
        }
        P.tick(PROF_SWEEP);
        if (cold) P.c[PROF_SWEEP_ICM] += clock64() - t_sw;
        const bool observe = A.obs != nullptr && D.hist_nbins > 0 && step >= A.hist_from;
        if (observe) {
            // magnetisation of the block's replicas, one warp per replica
            const int warp = tid >> 5, lane = tid & 31;
            for (int j = warp; j < rpc; j += (T >> 5)) {
                long long m = 0;
                for (int i = lane; i < n; i += 32) m += B.spin[(long long)j * npad + i];
                for (int o = 16; o > 0; o >>= 1) m += __shfl_xor_sync(0xffffffffu, m, o);
                if (lane == 0) s_mag[j] = m;
            }
            __syncthreads();
            if (D.group > 1)
                for (int j = tid; j < rpc; j += T)
                    A.mag_pub[parity * A.energy_pub_half + D.rep_off + B.r0 + j] = s_mag[j];
        }
        if (D.group > 1 && A.flag_barrier) {
            // publish this block's spins (for ICM partners), then each of its
            // replicas' energy tagged with this step in one 64-bit word,
            // stored with release; wait for every other replica's word of
            // this step, acquiring its block's spins with it.  No counter
            // to arrive at and no second hop: a block goes on as soon as the
            // last word it needs lands, holding the energies it read.
            if (icm_on) {
                const long long base = parity * A.spins_pub_half + D.spin_off + (long long)B.r0 * npad;
                for (int idx = tid; idx < rpc * npad; idx += T) A.spins_pub[base + idx] = B.spin[idx];
            }
            __syncthreads();
            unsigned long long* const ew = reinterpret_cast<unsigned long long*>(A.energy_pub) +
                                           (parity * A.energy_pub_half + D.rep_off) * kPubStride;
            const uint32_t tag = A.pub_base + (uint32_t)ls;
            for (int j = tid; j < rpc; j += T)
                st_release_gpu_u64(ew + (B.r0 + j) * kPubStride, pub_word(tag, B.E[B.r0 + j]));
            const unsigned long long limit = A.wait_limit_ns ? A.wait_limit_ns : kWaitLimitNs;
            int ok = 1;
            bool polled = false;
            for (int r = tid; r < R && ok; r += T) {
                if (r >= B.r0 && r < B.r0 + rpc) continue;
                polled = true;
                const unsigned long long t0 = globaltimer_ns();
                unsigned int spins = 0;
                unsigned long long w;
                while ((uint32_t)((w = ld_relaxed_gpu_u64(ew + r * kPubStride)) >> 32) != tag) {
                    if (*abortf) { ok = 0; break; }
                    if ((++spins & 63u) == 0 && globaltimer_ns() - t0 > limit) {
                        dev_fail(A.status, A.abort_flag, DEV_BARRIER_TIMEOUT, 1, blockIdx.x, tag);
                        ok = 0;
                        break;
                    }
                    __nanosleep(32);
                }
                if (ok) B.E[r] = (long long)(int32_t)(uint32_t)w;
            }
            if (A.bar_phantom && tid == 0 && ok) {
                // test hook: one more member whose word never comes
                const unsigned long long t0 = globaltimer_ns();
                while (ok) {
                    if (*abortf) ok = 0;
                    else if (globaltimer_ns() - t0 > limit) {
                        dev_fail(A.status, A.abort_flag, DEV_BARRIER_TIMEOUT, 1, blockIdx.x, tag);
                        ok = 0;
                    } else __nanosleep(256);
                }
            }
            // the words were read relaxed: each thread that read one acquires
            // what its release published (the block's barrier passes it on)
            if (polled) fence_acq_rel_gpu();
            if (!__syncthreads_and(ok)) break;
        } else if (D.group > 1) {
            // publish this block's energies (and spins, for ICM partners)
            for (int j = tid; j < rpc; j += T) A.energy_pub[parity * A.energy_pub_half + D.rep_off + B.r0 + j] = B.E[B.r0 + j];
            if (icm_on) {
                const long long base = parity * A.spins_pub_half + D.spin_off + (long long)B.r0 * npad;
                for (int idx = tid; idx < rpc * npad; idx += T) A.spins_pub[base + idx] = B.spin[idx];
            }
            if (!group_barrier(A.bar + 2 * inst, (unsigned)(D.group + A.bar_phantom), abortf, A.status, bar_gen,
                               A.wait_limit_ns ? A.wait_limit_ns : kWaitLimitNs))
                break;
            for (int r = tid; r < R; r += T)
                if (r < B.r0 || r >= B.r0 + rpc) B.E[r] = ld_cg(A.energy_pub + parity * A.energy_pub_half + D.rep_off + r);
            __syncthreads();
        }
        P.tick(PROF_BARRIER);
        if (A.hist != nullptr && D.hist_nbins > 0 && step >= A.hist_from && B.rank == 0) {
            for (int k = tid; k < R; k += T) {
                const int r = (int)B.slot[k];
                const long long bin = (B.E[r] - D.hist_lo) >> 1;
                if (bin >= 0 && bin < D.hist_nbins)
                    atomicAdd(A.hist + D.hist_off + (long long)k * D.hist_nbins + bin, 1u);
                if (observe) {
                    const long long m = (r >= B.r0 && r < B.r0 + rpc)
                                            ? s_mag[r - B.r0]
                                            : ld_cg(A.mag_pub + parity * A.energy_pub_half + D.rep_off + r);
                    unsigned long long* o = reinterpret_cast<unsigned long long*>(A.obs + 2 * (D.rep_off + k));
                    atomicAdd(o, (unsigned long long)m);
                    atomicAdd(o + 1, (unsigned long long)(m * m));
                }
            }
            __syncthreads();
        }
        if (A.phase_mask & PHASE_EXCHANGE) {
            if (REPLAY) exchange_replay(A, B, ls, s_beta, s_att, s_succ);
            else if (A.flags & ENGINE_EXCHANGE_EVEN_ODD) exchange_even_odd(A, B, step, s_dbeta, s_att, s_succ);
            else exchange_reference_order(A, B, step, s_order, s_dbeta, s_att, s_succ, s_xlogu, s_xrand, s_lvl, s_tmp, s_misc, P);
            for (int s = tid; s < R; s += T) {
                const uint32_t r = B.slot[s];
                if ((int)r >= B.r0 && (int)r < B.r0 + rpc) {
                    B.rslot[r - B.r0] = (uint32_t)s;
                    B.tb[r - B.r0] = (int)(((uint32_t)s % (uint32_t)nt) * (uint32_t)kst);
                }
            }
            __syncthreads();
        }
        P.tick(PROF_EXCHANGE);
        if (icm_on) {
            // pairs q = cp*nc + kk: slots (2cp)*nt + k and (2cp+1)*nt + k, k = nt-1-kk
            // the block's pairs, found from its own replicas' slots: replica
            // j at slot s (chain c = s / nt, temperature k = s % nt) is in pair
            // q = (c / 2) nc + (nt-1-k) when nt-1-k < nc; a pair with both
            // replicas in the block is taken from its first chain's side
            const int chains_even = D.chains & ~1;
            // the whole block is one team when it holds one replica, or when
            // the instance is configured with one team (large instances: a
            // pair per block-wide team, in sequence, beats a pair per warp)
            if (BLOCKTEAM || D.teams == 1) {
                const Team<true> team{tid, T, s_team_acc, s_team_bc};
                IcmScratch X = icm_scratch(s_icm, npad);
                if (!BLOCKTEAM && !REPLAY && S.icm_split)
                    X.list = reinterpret_cast<int*>(A.icm_pool + (size_t)blockIdx.x * (size_t)A.icm_pool_stride);
                for (int j = 0; j < rpc; j++) {
                    const int sl = (int)B.rslot[j], c = sl / nt, k = sl - c * nt, kk = nt - 1 - k;
                    if (kk >= D.nc || c >= chains_even) continue;
                    const int cp = c >> 1;
                    const int rA = (int)B.slot[(2 * cp) * nt + k], rB = (int)B.slot[(2 * cp + 1) * nt + k];
                    if ((c & 1) && rA >= B.r0 && rA < B.r0 + rpc) continue;
                    icm_pair<true, REPLAY, !REPLAY && (NARROW || !BLOCKTEAM), !REPLAY && !BLOCKTEAM>(
                                                                             A, B, team, cp * D.nc + kk, rA, rB,
                                                                             step, ls, X, 30, P);
                }
            } else {
                const int warp = tid >> 5, lane = tid & 31;
                const int teams = min(D.teams, T >> 5);
                if (warp < teams) {
                    Team<false> team{lane, 32, s_team_acc + warp, s_team_bc + 2 * warp};
                    const IcmScratch X = icm_scratch(s_icm + (size_t)warp * icm_team_bytes(npad), npad);
                    int e = 0;
                    for (int j = 0; j < rpc; j++) {
                        const int sl = (int)B.rslot[j], c = sl / nt, k = sl - c * nt, kk = nt - 1 - k;
                        if (kk >= D.nc || c >= chains_even) continue;
                        const int cp = c >> 1;
                        const int rA = (int)B.slot[(2 * cp) * nt + k], rB = (int)B.slot[(2 * cp + 1) * nt + k];
                        if ((c & 1) && rA >= B.r0 && rA < B.r0 + rpc) continue;
                        if ((e++ % teams) != warp) continue;
                        icm_pair<false, REPLAY, false>(A, B, team, cp * D.nc + kk, rA, rB, step, ls, X, 30, P);
                    }
                }
            }
            __syncthreads();
            // the block team's reduction slots back to the identity (the
            // next step's barriers publish it)
            if (tid == 0)
                for (int q = 0; q < 3; q++) team_slot_reset(s_team_acc, q);
        }
        P.tick(PROF_ICM);
    }
    __syncthreads();
    if (A.job_ns != nullptr && tid == 0 && A.nsteps > 1) A.job_ns[job] = globaltimer_ns() - t_step1;
    if (P.on) {
        P.c[PROF_TOTAL] = clock64() - t_start;
        for (int q = 0; q < PROF_PHASES; q++) A.prof[(size_t)blockIdx.x * PROF_PHASES + q] += (unsigned long long)P.c[q];
    }
    // ---- write the block's state back
    if (!S.state_global) {
        const long long base = D.spin_off + (long long)B.r0 * npad;
        for (int idx = tid; idx < rpc * npad; idx += T) {
            A.spins[base + idx] = B.spin[idx];
            if (B.field) A.fields[base + idx] = B.field[idx];
        }
        if (S.field_gather) {
            // the stored fields of the master copy, gathered once per launch
            for (int idx = tid; idx < rpc * npad; idx += T) {
                const int j = idx / npad, i = idx - j * npad;
                A.fields[base + idx] = i < n ? gather_field(B.row, B.adj, B.spin + (long long)j * npad, i) : 0;
            }
        }
    }
    for (int j = tid; j < rpc; j += T) {
        const long long g = D.rep_off + B.r0 + j;
        A.energy[g] = B.E[B.r0 + j];
        A.best_E[g] = s_bestE[j];
        A.flips[g] += s_flips[j];
    }
    if (B.rank == 0) {
        for (int r = tid; r < R; r += T) {
            A.slot_rep[D.rep_off + r] = B.slot[r];
            A.attempts[D.rep_off + r] += s_att[r];
            A.successes[D.rep_off + r] += s_succ[r];
        }
        for (int k = tid; k < nt; k += T) A.xorder[D.rep_off + k] = s_order[k];
    }
    // the next job restages shared memory
    __syncthreads();
    }
}

// --------------------------------------------------- from-scratch checks
// For every replica: fields f_i = sum_j J_ij s_j, E = sum h s + 1/2 sum s f
// and the cut sum over edges of w [s_i != s_j] (src/problem.cc:33-162),
// compared with the tracked fields and energy.  One block per replica.
__global__ void recompute_kernel(const EngineArgs A, const int32_t* rep_inst, int total_reps, int write_back,
                                 unsigned long long* mismatches, long long* E_out, long long* cut2_out) {
    const int g = blockIdx.x;
    if (g >= total_reps) return;
    const InstanceDesc D = A.desc[rep_inst[g]];
    const int r = (int)(g - D.rep_off);
    const int8_t* s = A.spins + D.spin_off + (long long)r * D.n_pad;
    int32_t* f = A.fields + D.spin_off + (long long)r * D.n_pad;
    const int32_t* row = A.row + D.row_off;
    const uint32_t* adj = A.adj + D.adj_off;
    long long e2 = 0, cut2 = 0;
    unsigned long long bad = 0;
    for (int i = threadIdx.x; i < D.n; i += blockDim.x) {
        int fi = 0;
        long long ci = 0;
        const int si = s[i];
        for (int a = row[i]; a < row[i + 1]; a++) {
            const uint32_t e = adj[a];
            const int J = (int)(int8_t)(e & 0xffu);
            const int sv = s[e >> 8];
            fi += J * sv;
            if (sv != si) ci += J;
        }
        const int hi = D.has_h ? A.hpool[D.h_off + i] : 0;
        e2 += (long long)si * (2 * hi + fi);
        cut2 += ci;
        if (si != 1 && si != -1) bad++;
        if (write_back) f[i] = fi;
        else if (f[i] != fi) bad++;
    }
    __shared__ long long red[3][32];
    for (int o = 16; o > 0; o >>= 1) {
        e2 += __shfl_xor_sync(0xffffffffu, e2, o);
        cut2 += __shfl_xor_sync(0xffffffffu, cut2, o);
        bad += __shfl_xor_sync(0xffffffffu, bad, o);
    }
    const int w = threadIdx.x >> 5, l = threadIdx.x & 31, nw = blockDim.x >> 5;
    if (l == 0) { red[0][w] = e2; red[1][w] = cut2; red[2][w] = (long long)bad; }
    __syncthreads();
    if (threadIdx.x == 0) {
        long long te = 0, tc = 0, tb = 0;
        for (int k = 0; k < nw; k++) { te += red[0][k]; tc += red[1][k]; tb += red[2][k]; }
        const long long E = te / 2;
        if (write_back) A.energy[g] = E;
        else if (A.energy[g] != E) tb++;
        if (E_out) E_out[g] = E;
        if (cut2_out) cut2_out[g] = tc;
        if (mismatches) atomicAdd(mismatches, (unsigned long long)tb);
    }
}

// Bernoulli(1/2) initial spins from the Philox init stream.
__global__ void init_spins_kernel(const EngineArgs A, const int32_t* rep_inst, int total_reps,
                                  unsigned long long seed) {
    const int g = blockIdx.x;
    if (g >= total_reps) return;
    const InstanceDesc D = A.desc[rep_inst[g]];
    const int r = (int)(g - D.rep_off);
    int8_t* s = A.spins + D.spin_off + (long long)r * D.n_pad;
    const uint2 key = stream_key(seed, STREAM_INIT);
    for (int i4 = threadIdx.x; i4 * 4 < D.n_pad; i4 += blockDim.x) {
        const uint4 x = philox4x32_10(make_uint4((uint32_t)i4, (uint32_t)r, (uint32_t)D.inst_id, 0x5EEDu), key);
        const uint32_t v[4] = {x.x, x.y, x.z, x.w};
#pragma unroll
        for (int q = 0; q < 4; q++) {
            const int i = i4 * 4 + q;
            if (i < D.n_pad) s[i] = (i < D.n) ? (int8_t)((v[q] >> 31) ? 1 : -1) : (int8_t)1;
        }
    }
}

// States given by the caller (R x n bytes, 0/1, original site order) into
// the device order as +-1 spins: replica r's site i goes to iperm[i];
// padding sites hold +1.
__global__ void load_states_kernel(const uint8_t* src, const int32_t* iperm, int8_t* spins, int R, int n, int n_pad) {
    const long long total = (long long)R * n_pad;
    for (long long idx = (long long)blockIdx.x * blockDim.x + threadIdx.x; idx < total;
         idx += (long long)gridDim.x * blockDim.x) {
        const int r = (int)(idx / n_pad), i = (int)(idx - (long long)r * n_pad);
        if (i < n) spins[(long long)r * n_pad + iperm[i]] = src[(long long)r * n + i] ? (int8_t)1 : (int8_t)-1;
        else spins[idx] = 1;
    }
}

// Philox outputs for host-side known-answer checks.
__global__ void philox_probe_kernel(const uint4* ctr, const uint2* key, uint4* out, int count) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i < count) out[i] = philox4x32_10(ctr[i], key[i]);
}

// Problem::energy / maxcut / calculate_dE for a batch of states (device
// order, +-1): E, twice the cut, and dE_i = -2 s_i (h_i + f_i).
__global__ void evaluate_kernel(const int32_t* row, const uint32_t* adj, const int32_t* h, int n, int n_pad,
                                const int8_t* states, int count, long long* E_out, long long* cut2_out,
                                int32_t* dE_out) {
    const int g = blockIdx.x;
    if (g >= count) return;
    const int8_t* s = states + (long long)g * n_pad;
    long long e2 = 0, cut2 = 0;
    for (int i = threadIdx.x; i < n; i += blockDim.x) {
        int fi = 0;
        long long ci = 0;
        const int si = s[i];
        for (int a = row[i]; a < row[i + 1]; a++) {
            const uint32_t e = adj[a];
            const int J = (int)(int8_t)(e & 0xffu);
            const int sv = s[e >> 8];
            fi += J * sv;
            if (sv != si) ci += J;
        }
        const int hi = h ? h[i] : 0;
        e2 += (long long)si * (2 * hi + fi);
        cut2 += ci;
        if (dE_out) dE_out[(long long)g * n_pad + i] = -2 * si * (hi + fi);
    }
    __shared__ long long red[2][32];
    for (int o = 16; o > 0; o >>= 1) {
        e2 += __shfl_xor_sync(0xffffffffu, e2, o);
        cut2 += __shfl_xor_sync(0xffffffffu, cut2, o);
    }
    const int w = threadIdx.x >> 5, l = threadIdx.x & 31, nw = blockDim.x >> 5;
    if (l == 0) { red[0][w] = e2; red[1][w] = cut2; }
    __syncthreads();
    if (threadIdx.x == 0) {
        long long te = 0, tc = 0;
        for (int k = 0; k < nw; k++) { te += red[0][k]; tc += red[1][k]; }
        E_out[g] = te / 2;
        cut2_out[g] = tc;
    }
}

// ------------------------------------------------------------ launchers
static void* engine_fn(bool replay, bool block_team, bool narrow) {
    if (replay) return (void*)pt_engine_kernel<true, false, false>;
    if (block_team && narrow) return (void*)pt_engine_kernel<false, true, true>;
    if (block_team) return (void*)pt_engine_kernel<false, true, false>;
    return (void*)pt_engine_kernel<false, false, false>;
}

// Tags of published energy words: one per PT step of every launch in the
// process, never 0 (a zeroed word) and never repeated within 2^32 steps.
static std::atomic<uint32_t> g_pub_tag{1u};

cudaError_t launch_engine(const EngineArgs& A0, int threads, bool replay, bool block_team, bool narrow,
                          bool cooperative, cudaStream_t stream) {
    void* fn = engine_fn(replay, block_team, narrow);
    cudaError_t e = cudaFuncSetAttribute(fn, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)A0.sm.total);
    if (e != cudaSuccess) return e;
    EngineArgs A = A0;
    const uint32_t span = (uint32_t)std::max(A.nsteps, 1) + 1u;
    uint32_t base = g_pub_tag.fetch_add(span);
    if (base == 0u || base + span < base) base = g_pub_tag.fetch_add(span);   // (past the wrap: 0 stays unused)
    A.pub_base = base;
    void* args[] = {(void*)&A};
    if (cooperative)
        return cudaLaunchCooperativeKernel(fn, dim3(A.n_blocks), dim3(threads), args, A.sm.total, stream);
    return cudaLaunchKernel(fn, dim3(A.n_blocks), dim3(threads), args, A.sm.total, stream);
}

cudaError_t engine_max_blocks_per_sm(bool replay, bool block_team, bool narrow, int threads, size_t smem, int* out) {
    if (!replay && (narrow || !block_team) && threads > kNarrowThreads) {
        *out = 0;
        return cudaSuccess;
    }
    const void* fn = engine_fn(replay, block_team, narrow);
    cudaError_t e = cudaFuncSetAttribute(fn, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
    if (e != cudaSuccess) return e;
    return cudaOccupancyMaxActiveBlocksPerMultiprocessor(out, fn, threads, smem);
}

cudaError_t launch_recompute(const EngineArgs& A, const int32_t* rep_inst, int total_reps, int write_back,
                             unsigned long long* mismatches, long long* E_out, long long* cut2_out,
                             cudaStream_t stream) {
    recompute_kernel<<<total_reps, 256, 0, stream>>>(A, rep_inst, total_reps, write_back, mismatches, E_out, cut2_out);
    return cudaGetLastError();
}

cudaError_t launch_init_spins(const EngineArgs& A, const int32_t* rep_inst, int total_reps,
                              unsigned long long seed, cudaStream_t stream) {
    init_spins_kernel<<<total_reps, 256, 0, stream>>>(A, rep_inst, total_reps, seed);
    return cudaGetLastError();
}

cudaError_t launch_load_states(const uint8_t* src, const int32_t* iperm, int8_t* spins, int R, int n, int n_pad,
                               cudaStream_t stream) {
    const long long total = (long long)R * n_pad;
    const int blocks = (int)std::min<long long>((total + 255) / 256, 4096);
    load_states_kernel<<<blocks, 256, 0, stream>>>(src, iperm, spins, R, n, n_pad);
    return cudaGetLastError();
}

cudaError_t launch_evaluate(const int32_t* row, const uint32_t* adj, const int32_t* h, int n, int n_pad,
                            const int8_t* states, int count, long long* E_out, long long* cut2_out,
                            int32_t* dE_out, cudaStream_t stream) {
    evaluate_kernel<<<count, 256, 0, stream>>>(row, adj, h, n, n_pad, states, count, E_out, cut2_out, dE_out);
    return cudaGetLastError();
}

cudaError_t launch_philox_probe(const uint4* ctr, const uint2* key, uint4* out, int count, cudaStream_t stream) {
    philox_probe_kernel<<<(count + 127) / 128, 128, 0, stream>>>(ctr, key, out, count);
    return cudaGetLastError();
}

}  // namespace pticm
