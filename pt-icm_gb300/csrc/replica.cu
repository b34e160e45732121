// replica.cu -- single replicas and single ICM pairs on the GPU: the
// per-replica, per-pair layer of the reference's libreplica interface
// (include/replica.hh, include/icm.hh, Problem::incremental_dE), for code
// written in the reference's shape (its solve loop, src/solver.cc:67-127, and
// the pilot loop of get_beta, src/cae_estimator.cc:112-140).
//
// A pticm_replica is one replica in device memory: int8 spins and int32 local
// fields in the engine's site order, its energy, its best energy and state,
// flip and sweep counters, and the FP64 table exp(-beta dE) of its
// temperature.  A sweep is the reference's sequential Metropolis sweep
// (src/replica.cc:5-38) with the uniforms the caller draws from its own
// generator: the caller passes enough of them (one per site at most) and
// learns how many the sweep consumed, so that its generator stays in step
// with the reference's.  The bulk PT path (pticm_run) does not use this file.
#include <cuda_runtime.h>

#include <algorithm>
#include <cmath>
#include <memory>
#include <string>
#include <vector>

#include "pticm.h"
#include "pticm_device.cuh"
#include "pticm_engine.h"
#include "runtime_internal.h"

using namespace pticm;

struct pticm_replica {
    const pticm_problem* p = nullptr;
    ProblemDevice P{};
    double beta = 0.0;
    bool log_energy = false;
    uint64_t burn_in = 0;
    DArr<int8_t> s, best;         // spins and best state (device order, n_pad)
    DArr<int32_t> f;              // local fields f_i = sum_j J_ij s_j
    DArr<long long> e;            // energy, best energy
    DArr<unsigned long long> c;   // best sweep, flips, sweeps
    DArr<double> ptab;            // exp(-beta * 2t), t = 0..kmax
    DArr<double> u;               // the caller's uniforms of one sweep (n)
    DArr<long long> elog;         // energies after every site (log_energy)
    DArr<unsigned long long> used;
    DArr<int> status;
};

namespace {

int rfail(int code, const std::string& m) {
    set_last_error(m);
    return code;
}

#define R_CK(x)                                                                                        \
    do {                                                                                               \
        cudaError_t e_ = (x);                                                                          \
        if (e_ != cudaSuccess) return rfail(PTICM_ERR_CUDA, std::string(#x) + ": " + cudaGetErrorString(e_)); \
    } while (0)

// Caller states (0/1 bytes, original order) into device order +-1 spins; the
// padding sites hold +1.
__global__ void rep_import(const uint8_t* src, const int32_t* iperm, int8_t* s, int n, int n_pad) {
    for (int i = threadIdx.x; i < n; i += blockDim.x) s[iperm[i]] = src[i] ? (int8_t)1 : (int8_t)-1;
}

__global__ void rep_pad(int8_t* s, int n, int n_pad) {
    for (int i = n + threadIdx.x; i < n_pad; i += blockDim.x) s[i] = 1;
}

// Local fields and energy from scratch (Problem::calculate_dE,
// src/problem.cc:33-63, in integers): f_i = sum_j J_ij s_j and
// E = sum_i s_i (h_i + f_i / 2).  One block.
__global__ void rep_fields(const int32_t* row, const uint32_t* adj, const int32_t* h, int n, const int8_t* s,
                           int32_t* f, long long* E) {
    long long e2 = 0;
    for (int i = threadIdx.x; i < n; i += blockDim.x) {
        int fi = 0;
        for (int a = row[i]; a < row[i + 1]; a++) {
            const uint32_t x = adj[a];
            fi += (int)(int8_t)(x & 0xffu) * s[x >> 8];
        }
        f[i] = fi;
        e2 += (long long)s[i] * (2 * (h ? h[i] : 0) + fi);
    }
    __shared__ long long red[32];
    for (int o = 16; o > 0; o >>= 1) e2 += __shfl_xor_sync(0xffffffffu, e2, o);
    if ((threadIdx.x & 31) == 0) red[threadIdx.x >> 5] = e2;
    __syncthreads();
    if (threadIdx.x == 0) {
        long long t = 0;
        for (int w = 0; w < (int)(blockDim.x >> 5); w++) t += red[w];
        *E = t / 2;
    }
}

// Replica::sweep (src/replica.cc:5-38): the sites in the reference's order
// 0..n-1 (device site iperm[o]); lane 0 decides each move exactly as
// mh_consider does (dE <= 0, else u < exp(-beta dE) with the next caller
// uniform), the warp pushes the field change of an accepted flip and copies a
// new best state (mh_accept).  e[0] energy, e[1] best energy; c[0] best sweep,
// c[1] flips, c[2] sweeps.  One warp.
__global__ void rep_sweep(const int32_t* row, const uint32_t* adj, const int32_t* h, const int32_t* iperm, int n,
                          int n_pad, int kmax, const double* ptab, int8_t* s, int32_t* f, long long* e,
                          unsigned long long* c, int8_t* best, const double* u, unsigned long long nu,
                          unsigned long long* used, long long* elog, int* status) {
    const int lane = threadIdx.x;
    long long E = e[0], bestE = e[1];
    const unsigned long long sweep = c[2];
    unsigned long long pos = 0, flips = 0;
    int bad = 0;
    for (int o = 0; o < n; o++) {
        const int i = iperm[o];
        int acc = 0, si = 0, de = 0;
        if (lane == 0) {
            si = s[i];
            de = -2 * si * (f[i] + (h ? h[i] : 0));
            if (de <= 0) {
                acc = 1;
            } else if (pos < nu) {
                acc = u[pos++] < ptab[min(de >> 1, kmax)];
            } else {
                bad = 1;
            }
        }
        acc = __shfl_sync(0xffffffffu, acc, 0);
        if (acc) {
            si = __shfl_sync(0xffffffffu, si, 0);
            de = __shfl_sync(0xffffffffu, de, 0);
            for (int a = row[i] + lane; a < row[i + 1]; a += 32) {
                const uint32_t x = adj[a];
                atomicAdd(f + (x >> 8), (int)(int8_t)(x & 0xffu) * (-2 * si));   // parallel edges
            }
            __syncwarp();
            if (lane == 0) s[i] = (int8_t)-si;
            E += de;
            flips++;
            if (E < bestE) {
                bestE = E;
                __syncwarp();
                for (int x = lane; x < n_pad; x += 32) best[x] = s[x];
                if (lane == 0) c[0] = sweep;
            }
            __syncwarp();
        }
        if (elog && lane == 0) elog[o] = E;
    }
    if (lane == 0) {
        e[0] = E;
        e[1] = bestE;
        c[1] += flips;
        c[2] = sweep + 1;
        *used = pos;
        *status = bad;
    }
}

// xor_icm's overlap (src/icm.cc:8-31) on caller states in the original order:
// count the differing sites; when more than n/2 differ, negate s1 first;
// write the differing sites ascending.  One block of 1024 threads.
__global__ void pair_overlap(uint8_t* s1, const uint8_t* s2, int n, long long* sites, long long* count) {
    __shared__ int warp_tot[32];
    __shared__ long long base;
    int local = 0;
    for (int i = threadIdx.x; i < n; i += blockDim.x) local += (s1[i] != 0) != (s2[i] != 0);
    for (int o = 16; o > 0; o >>= 1) local += __shfl_xor_sync(0xffffffffu, local, o);
    if ((threadIdx.x & 31) == 0) warp_tot[threadIdx.x >> 5] = local;
    __syncthreads();
    long long cnt = 0;
    for (int w = 0; w < (int)(blockDim.x >> 5); w++) cnt += warp_tot[w];
    __syncthreads();
    const bool gflip = cnt > (long long)(n / 2);
    if (gflip)
        for (int i = threadIdx.x; i < n; i += blockDim.x) s1[i] = s1[i] ? 0 : 1;
    else
        for (int i = threadIdx.x; i < n; i += blockDim.x) s1[i] = s1[i] ? 1 : 0;
    if (threadIdx.x == 0) base = 0;
    __syncthreads();
    // ascending compaction, one chunk of blockDim sites at a time
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    for (int c0 = 0; c0 < n; c0 += blockDim.x) {
        const int i = c0 + threadIdx.x;
        const bool d = i < n && (s1[i] != (s2[i] != 0));
        const unsigned m = __ballot_sync(0xffffffffu, d);
        if (lane == 0) warp_tot[warp] = __popc(m);
        __syncthreads();
        long long off = base;
        for (int w = 0; w < warp; w++) off += warp_tot[w];
        if (d) sites[off + __popc(m & ((1u << lane) - 1u))] = i;
        __syncthreads();
        if (threadIdx.x == 0)
            for (int w = 0; w < (int)(blockDim.x >> 5); w++) base += warp_tot[w];
        __syncthreads();
    }
    if (threadIdx.x == 0) *count = base;
}

// bfs_icm (src/icm.cc:37-72) on device-order states: the seed's connected
// set of differing sites (grown level by level; the reference grows it
// depth-first, which finds the same set) is flipped in both states.  `queue`
// holds n ints, `vis` (n + 31) / 32 zeroed words.  One block.
__global__ void pair_cluster(const int32_t* row, const uint32_t* adj, int8_t* s1, int8_t* s2, int seed,
                             int* queue, unsigned* vis, int* status) {
    __shared__ int tail;
    const int lane = threadIdx.x & 31;
    if (threadIdx.x == 0) {
        queue[0] = seed;
        vis[seed >> 5] |= 1u << (seed & 31);
        tail = 1;
        *status = (s1[seed] == s2[seed]) ? 1 : 0;
    }
    __syncthreads();
    int lo = 0;
    while (true) {
        const int hi = *(volatile int*)&tail;
        __syncthreads();
        if (lo == hi) break;
        for (int b = lo; b < hi; b += blockDim.x) {
            const int idx = b + threadIdx.x;
            const bool have = idx < hi;
            const int uu = have ? queue[idx] : 0;
            const int e0 = have ? row[uu] : 0, deg = have ? row[uu + 1] - e0 : 0;
            for (int k = 0; __any_sync(0xffffffffu, k < deg); k++) {
                bool found = false;
                int v = 0;
                if (k < deg) {
                    v = (int)(adj[e0 + k] >> 8);
                    if (s1[v] != s2[v]) {
                        const unsigned bit = 1u << (v & 31);
                        found = !(atomicOr(vis + (v >> 5), bit) & bit);
                    }
                }
                const unsigned m = __ballot_sync(0xffffffffu, found);
                if (m) {
                    const int leader = __ffs(m) - 1;
                    int slot = 0;
                    if (lane == leader) slot = atomicAdd(&tail, __popc(m));
                    slot = __shfl_sync(0xffffffffu, slot, leader);
                    if (found) queue[slot + __popc(m & ((1u << lane) - 1u))] = v;
                }
            }
        }
        __syncthreads();
        lo = hi;
    }
    for (int t = threadIdx.x; t < lo; t += blockDim.x) {
        const int v = queue[t];
        s1[v] = (int8_t)-s1[v];
        s2[v] = (int8_t)-s2[v];
    }
}

// Problem::incremental_dE (src/problem.cc:164-181) on a caller dE vector in
// the original order, with the state before site `index` flips:
// dE[index] = -dE[index]; dE[j] += 4 s_index s_j J_index,j.
__global__ void incremental_dE_kernel(const int32_t* row, const uint32_t* adj, const int32_t* perm, int d,
                                      double* dE, const uint8_t* s, int index) {
    const int si = s[index] ? 1 : -1;
    for (int a = row[d] + threadIdx.x; a < row[d + 1]; a += blockDim.x) {
        const uint32_t x = adj[a];
        const int j = perm[x >> 8];
        const int sj = s[j] ? 1 : -1;
        atomicAdd(dE + j, (double)(4 * si * sj * (int)(int8_t)(x & 0xffu)));   // exact integers: any order
    }
    if (threadIdx.x == 0) dE[index] = -dE[index];
}

int upload_ptab(pticm_replica* r) {
    std::vector<double> t((size_t)r->P.kmax + 1, 1.0);
    for (int k = 1; k <= r->P.kmax; k++) t[k] = std::exp(-r->beta * (2.0 * k));   // src/replica.cc:35
    R_CK(cudaMemcpy(r->ptab.p, t.data(), t.size() * sizeof(double), cudaMemcpyHostToDevice));
    return PTICM_OK;
}

int load_state(pticm_replica* r, const uint8_t* state) {
    DArr<uint8_t> tmp;
    R_CK(tmp.alloc((size_t)std::max(r->P.n, 1)));
    R_CK(cudaMemcpy(tmp.p, state, (size_t)r->P.n, cudaMemcpyHostToDevice));
    rep_pad<<<1, 256>>>(r->s.p, r->P.n, r->P.n_pad);
    rep_import<<<1, 1024>>>(tmp.p, r->P.iperm, r->s.p, r->P.n, r->P.n_pad);
    rep_fields<<<1, 1024>>>(r->P.row, r->P.adj, r->P.has_h ? r->P.h : nullptr, r->P.n, r->s.p, r->f.p, r->e.p);
    R_CK(cudaGetLastError());
    R_CK(cudaDeviceSynchronize());
    return PTICM_OK;
}

// host states (original order) <-> device order for the pair calls
std::vector<int8_t> to_device_order(const HostProblem& P, const uint8_t* s) {
    std::vector<int8_t> d((size_t)pad16(P.n), 1);
    for (int64_t i = 0; i < P.n; i++) d[(size_t)P.iperm[i]] = s[i] ? 1 : -1;
    return d;
}

}  // namespace

extern "C" {

int pticm_replica_create(const pticm_problem* p, double beta, const uint8_t* state, pticm_replica** out) {
    if (!p || !state || !out) return rfail(PTICM_ERR_INVALID, "null argument");
    if (!std::isfinite(beta)) return rfail(PTICM_ERR_INVALID, "non-finite inverse temperature");
    int count = 0;
    if (cudaGetDeviceCount(&count) != cudaSuccess || count == 0)
        return rfail(PTICM_ERR_NODEVICE, "no CUDA device is available; the PT-ICM engine has no CPU path");
    auto r = std::make_unique<pticm_replica>();
    r->p = p;
    if (int rc = problem_device(p, &r->P)) return rc;
    r->beta = beta;
    const size_t np = (size_t)std::max(r->P.n_pad, 16);
    R_CK(r->s.alloc(np));
    R_CK(r->best.alloc(np));
    R_CK(r->f.alloc(np));
    R_CK(r->e.alloc(2));
    R_CK(r->c.alloc(3));
    R_CK(r->ptab.alloc((size_t)r->P.kmax + 1));
    R_CK(r->u.alloc((size_t)std::max(r->P.n, 1)));
    R_CK(r->used.alloc(1));
    R_CK(r->status.alloc(1));
    if (int rc = upload_ptab(r.get())) return rc;
    if (int rc = load_state(r.get(), state)) return rc;
    // Replica(...) src/replica.cc:40-60: best energy "none yet", best state the initial one
    const long long none = kNoBest;
    R_CK(cudaMemcpy(r->e.p + 1, &none, sizeof none, cudaMemcpyHostToDevice));
    R_CK(cudaMemcpy(r->best.p, r->s.p, np, cudaMemcpyDeviceToDevice));
    *out = r.release();
    return PTICM_OK;
}

void pticm_replica_destroy(pticm_replica* r) { delete r; }

int pticm_replica_copy(const pticm_replica* src, pticm_replica** out) {
    if (!src || !out) return rfail(PTICM_ERR_INVALID, "null argument");
    std::vector<uint8_t> zero((size_t)std::max<int64_t>(src->P.n, 1), 0);
    pticm_replica* r = nullptr;
    if (int rc = pticm_replica_create(src->p, src->beta, zero.data(), &r)) return rc;
    std::unique_ptr<pticm_replica> hold(r);
    r->log_energy = src->log_energy;
    r->burn_in = src->burn_in;
    const size_t np = src->s.n;
    R_CK(cudaMemcpy(r->s.p, src->s.p, np, cudaMemcpyDeviceToDevice));
    R_CK(cudaMemcpy(r->best.p, src->best.p, np, cudaMemcpyDeviceToDevice));
    R_CK(cudaMemcpy(r->f.p, src->f.p, np * 4, cudaMemcpyDeviceToDevice));
    R_CK(cudaMemcpy(r->e.p, src->e.p, 2 * sizeof(long long), cudaMemcpyDeviceToDevice));
    R_CK(cudaMemcpy(r->c.p, src->c.p, 3 * sizeof(unsigned long long), cudaMemcpyDeviceToDevice));
    *out = hold.release();
    return PTICM_OK;
}

int pticm_replica_set_beta(pticm_replica* r, double beta) {
    if (!r) return rfail(PTICM_ERR_INVALID, "null argument");
    if (!std::isfinite(beta)) return rfail(PTICM_ERR_INVALID, "non-finite inverse temperature");
    if (beta == r->beta) return PTICM_OK;
    r->beta = beta;
    return upload_ptab(r);
}

int pticm_replica_set_state(pticm_replica* r, const uint8_t* state) {
    if (!r || !state) return rfail(PTICM_ERR_INVALID, "null argument");
    return load_state(r, state);
}

int pticm_replica_set_energy(pticm_replica* r, double energy) {
    if (!r) return rfail(PTICM_ERR_INVALID, "null argument");
    if (!(std::fabs(energy) < 9.0e18) || energy != std::floor(energy))
        return rfail(PTICM_ERR_UNSUPPORTED, "energies of integer couplings are integers");
    const long long e = (long long)energy;
    R_CK(cudaMemcpy(r->e.p, &e, sizeof e, cudaMemcpyHostToDevice));
    return PTICM_OK;
}

int pticm_replica_set_logging(pticm_replica* r, int log_energy, uint64_t burn_in) {
    if (!r) return rfail(PTICM_ERR_INVALID, "null argument");
    r->log_energy = log_energy != 0;
    r->burn_in = burn_in;
    if (r->log_energy && r->elog.n < (size_t)std::max(r->P.n, 1)) R_CK(r->elog.alloc((size_t)std::max(r->P.n, 1)));
    return PTICM_OK;
}

int pticm_replica_sweep(pticm_replica* r, const double* uniforms, uint64_t n_uniforms, uint64_t* consumed,
                        double* energy, double* energy_log) {
    if (!r || (n_uniforms && !uniforms)) return rfail(PTICM_ERR_INVALID, "null argument");
    const uint64_t nu = std::min<uint64_t>(n_uniforms, (uint64_t)r->P.n);
    if (nu) R_CK(cudaMemcpy(r->u.p, uniforms, nu * sizeof(double), cudaMemcpyHostToDevice));
    unsigned long long sweeps = 0;
    R_CK(cudaMemcpy(&sweeps, r->c.p + 2, sizeof sweeps, cudaMemcpyDeviceToHost));
    // log the energy after every site while logging and past the burn-in
    // (src/replica.cc:10-12: sweep_counter > burn_in)
    const bool logging = r->log_energy && sweeps > r->burn_in && energy_log;
    rep_sweep<<<1, 32>>>(r->P.row, r->P.adj, r->P.has_h ? r->P.h : nullptr, r->P.iperm, r->P.n, r->P.n_pad,
                         r->P.kmax, r->ptab.p, r->s.p, r->f.p, r->e.p, r->c.p, r->best.p, r->u.p, nu, r->used.p,
                         logging ? r->elog.p : nullptr, r->status.p);
    R_CK(cudaGetLastError());
    unsigned long long used = 0;
    int st = 0;
    long long e = 0;
    R_CK(cudaMemcpy(&used, r->used.p, sizeof used, cudaMemcpyDeviceToHost));
    R_CK(cudaMemcpy(&st, r->status.p, sizeof st, cudaMemcpyDeviceToHost));
    R_CK(cudaMemcpy(&e, r->e.p, sizeof e, cudaMemcpyDeviceToHost));
    if (st) return rfail(PTICM_ERR_INVALID, "the sweep needed more uniforms than were passed");
    if (consumed) *consumed = used;
    if (energy) *energy = (double)e;
    if (logging) {
        std::vector<long long> l((size_t)r->P.n);
        R_CK(cudaMemcpy(l.data(), r->elog.p, l.size() * sizeof(long long), cudaMemcpyDeviceToHost));
        for (size_t k = 0; k < l.size(); k++) energy_log[k] = (double)l[k];
    }
    return PTICM_OK;
}

int pticm_replica_get(pticm_replica* r, pticm_replica_info* info, uint8_t* state, double* dE, uint8_t* best_state) {
    if (!r) return rfail(PTICM_ERR_INVALID, "null argument");
    const HostProblem& P = problem_host(r->p);
    const int n = (int)P.n;
    if (info) {
        long long e[2];
        unsigned long long c[3];
        R_CK(cudaMemcpy(e, r->e.p, sizeof e, cudaMemcpyDeviceToHost));
        R_CK(cudaMemcpy(c, r->c.p, sizeof c, cudaMemcpyDeviceToHost));
        info->energy = (double)e[0];
        info->best_energy = e[1] == kNoBest ? 1.7976931348623157e308 : (double)e[1];
        info->beta = r->beta;
        info->best_sweep = c[0];
        info->flips = c[1];
        info->sweeps = c[2];
    }
    std::vector<int8_t> s;
    if (state || dE) {
        s.resize(r->s.n);
        R_CK(cudaMemcpy(s.data(), r->s.p, s.size(), cudaMemcpyDeviceToHost));
    }
    if (state)
        for (int i = 0; i < n; i++) state[i] = s[(size_t)P.iperm[i]] > 0 ? 1 : 0;
    if (dE) {
        std::vector<int32_t> f(r->f.n);
        R_CK(cudaMemcpy(f.data(), r->f.p, f.size() * 4, cudaMemcpyDeviceToHost));
        for (int i = 0; i < n; i++) {
            const size_t d = (size_t)P.iperm[i];
            dE[i] = (double)(-2 * s[d] * (f[d] + (P.has_h ? P.dh[d] : 0)));
        }
    }
    if (best_state) {
        std::vector<int8_t> b(r->best.n);
        R_CK(cudaMemcpy(b.data(), r->best.p, b.size(), cudaMemcpyDeviceToHost));
        for (int i = 0; i < n; i++) best_state[i] = b[(size_t)P.iperm[i]] > 0 ? 1 : 0;
    }
    return PTICM_OK;
}

int pticm_problem_icm_overlap(const pticm_problem* p, uint8_t* s1, const uint8_t* s2, uint64_t* count,
                              int64_t* sites) {
    if (!p || !s1 || !s2 || !count) return rfail(PTICM_ERR_INVALID, "null argument");
    int dc = 0;
    if (cudaGetDeviceCount(&dc) != cudaSuccess || dc == 0)
        return rfail(PTICM_ERR_NODEVICE, "no CUDA device is available; the PT-ICM engine has no CPU path");
    const int n = (int)problem_host(p).n;
    DArr<uint8_t> a, b;
    DArr<long long> st, cnt;
    R_CK(a.alloc((size_t)std::max(n, 1)));
    R_CK(b.alloc((size_t)std::max(n, 1)));
    R_CK(st.alloc((size_t)std::max(n, 1)));
    R_CK(cnt.alloc(1));
    R_CK(cudaMemcpy(a.p, s1, (size_t)n, cudaMemcpyHostToDevice));
    R_CK(cudaMemcpy(b.p, s2, (size_t)n, cudaMemcpyHostToDevice));
    pair_overlap<<<1, 1024>>>(a.p, b.p, n, st.p, cnt.p);
    R_CK(cudaGetLastError());
    long long c = 0;
    R_CK(cudaMemcpy(&c, cnt.p, sizeof c, cudaMemcpyDeviceToHost));
    R_CK(cudaMemcpy(s1, a.p, (size_t)n, cudaMemcpyDeviceToHost));
    if (sites && c) R_CK(cudaMemcpy(sites, st.p, (size_t)c * sizeof(long long), cudaMemcpyDeviceToHost));
    *count = (uint64_t)c;
    return PTICM_OK;
}

int pticm_problem_icm_cluster(const pticm_problem* p, int64_t seed, uint8_t* s1, uint8_t* s2) {
    if (!p || !s1 || !s2) return rfail(PTICM_ERR_INVALID, "null argument");
    const HostProblem& P = problem_host(p);
    if (seed < 0 || seed >= P.n) return rfail(PTICM_ERR_INVALID, "seed site out of range");
    ProblemDevice PD;
    if (int rc = problem_device(p, &PD)) return rc;
    const int n = (int)P.n, npad = pad16(P.n);
    std::vector<int8_t> a = to_device_order(P, s1), b = to_device_order(P, s2);
    DArr<int8_t> da, db;
    DArr<int> q, st;
    DArr<unsigned> vis;
    R_CK(da.upload(a));
    R_CK(db.upload(b));
    R_CK(q.alloc((size_t)npad));
    R_CK(vis.alloc((size_t)(npad + 31) / 32));
    R_CK(st.alloc(1));
    pair_cluster<<<1, 1024>>>(PD.row, PD.adj, da.p, db.p, P.iperm[seed], q.p, vis.p, st.p);
    R_CK(cudaGetLastError());
    int bad = 0;
    R_CK(cudaMemcpy(&bad, st.p, sizeof bad, cudaMemcpyDeviceToHost));
    if (bad) return rfail(PTICM_ERR_INVALID, "the seed is not a site where the two states differ");
    R_CK(da.download(a));
    R_CK(db.download(b));
    for (int i = 0; i < n; i++) {
        s1[i] = a[(size_t)P.iperm[i]] > 0 ? 1 : 0;
        s2[i] = b[(size_t)P.iperm[i]] > 0 ? 1 : 0;
    }
    return PTICM_OK;
}

int pticm_problem_incremental_dE(const pticm_problem* p, double* dE, const uint8_t* state, uint32_t index) {
    if (!p || !dE || !state) return rfail(PTICM_ERR_INVALID, "null argument");
    const HostProblem& P = problem_host(p);
    if ((int64_t)index >= P.n) return rfail(PTICM_ERR_INVALID, "site index out of range");
    ProblemDevice PD;
    if (int rc = problem_device(p, &PD)) return rc;
    const int n = (int)P.n;
    DArr<double> d;
    DArr<uint8_t> s;
    R_CK(d.alloc((size_t)n));
    R_CK(s.alloc((size_t)n));
    R_CK(cudaMemcpy(d.p, dE, (size_t)n * sizeof(double), cudaMemcpyHostToDevice));
    R_CK(cudaMemcpy(s.p, state, (size_t)n, cudaMemcpyHostToDevice));
    incremental_dE_kernel<<<1, 256>>>(PD.row, PD.adj, PD.perm, P.iperm[index], d.p, s.p, (int)index);
    R_CK(cudaGetLastError());
    R_CK(cudaMemcpy(dE, d.p, (size_t)n * sizeof(double), cudaMemcpyDeviceToHost));
    return PTICM_OK;
}

}  // extern "C"
