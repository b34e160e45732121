// pticm_device.cuh -- device-side building blocks shared by the PT-ICM kernels
// (sm_103a): counter-based RNG, bounded waits, bulk-copy staging, error words.
#pragma once
#include <cstdint>
#include <cuda_runtime.h>

#include "pticm_engine.h"

namespace pticm {

// ------------------------------------------------------------------ errors
// Device-side failures are recorded in one DevStatus word block; the first
// failure wins.  Kernels never trap: they record, raise `abort`, and return.
enum DevErr : int {
    DEV_OK = 0,
    DEV_BARRIER_TIMEOUT = 1,   // a group barrier waited longer than its limit
    DEV_TMA_TIMEOUT = 2,       // a bulk-copy mbarrier never completed
    DEV_UF_LIMIT = 3,          // cluster labelling did not converge within its round cap
    DEV_REPLAY_MISMATCH = 4,   // a replay trace disagrees with the device state
    DEV_BAD_INDEX = 5,         // an index failed a bounds check
    DEV_ABORTED = 6,           // another block aborted first
};

__device__ __forceinline__ void dev_fail(DevStatus* st, volatile int* abort_flag, int err, int where,
                                         long long a0 = 0, long long a1 = 0) {
    if (atomicCAS(&st->error, 0, err) == 0) {
        st->where = where;
        st->aux0 = a0;
        st->aux1 = a1;
    }
    *abort_flag = 1;
    __threadfence();
}

__device__ __forceinline__ unsigned long long globaltimer_ns() {
    unsigned long long t;
    asm volatile("mov.u64 %0, %%globaltimer;" : "=l"(t));
    return t;
}

// Waits on other blocks give up after this many nanoseconds (the default of
// EngineArgs::wait_limit_ns).
constexpr unsigned long long kWaitLimitNs = 2000000000ull;

// --------------------------------------------------------------------- RNG
// Philox4x32-10 (Salmon, Moraes, Dror, Shaw, "Parallel random numbers: as
// easy as 1, 2, 3", SC'11): ten rounds of two 32x32->64 multiplies with
// Weyl-sequence key increments.
__device__ __forceinline__ uint4 philox4x32_10(uint4 c, uint2 k) {
#pragma unroll
    for (int r = 0; r < 10; r++) {
        const uint32_t lo0 = 0xD2511F53u * c.x, hi0 = __umulhi(0xD2511F53u, c.x);
        const uint32_t lo1 = 0xCD9E8D57u * c.z, hi1 = __umulhi(0xCD9E8D57u, c.z);
        c = make_uint4(hi1 ^ c.y ^ k.x, lo1, hi0 ^ c.w ^ k.y, lo0);
        k.x += 0x9E3779B9u;
        k.y += 0xBB67AE85u;
    }
    return c;
}

// Independent Philox streams are separated by key: the run seed XOR a
// per-purpose constant.
enum StreamTag : uint32_t {
    STREAM_SWEEP = 0x00000000u,
    STREAM_EXCHANGE = 0x45584348u,  // "EXCH"
    STREAM_ICM = 0x49434D31u,       // "ICM1"
    STREAM_INIT = 0x494E4954u,      // "INIT"
};

__device__ __forceinline__ uint2 stream_key(unsigned long long seed, uint32_t tag) {
    return make_uint2((uint32_t)seed ^ tag, (uint32_t)(seed >> 32) ^ (tag * 0x9E3779B9u));
}

// A per-thread buffered Philox stream: four 32-bit words per block call.
struct ThreadRng {
    uint4 buf;
    uint32_t avail;
    uint32_t calls;
    uint4 ctr;   // (thread id, step lo, step hi, call index)
    uint2 key;

    __device__ __forceinline__ void start(uint2 k, uint32_t tid, unsigned long long step) {
        key = k;
        ctr = make_uint4(tid, (uint32_t)step, (uint32_t)(step >> 32), 0u);
        avail = 0;
        calls = 0;
    }
    __device__ __forceinline__ uint32_t next() {
        if (avail == 0) {
            ctr.w = calls++;
            buf = philox4x32_10(ctr, key);
            avail = 4;
        }
        const uint32_t r = buf.x;
        buf.x = buf.y;
        buf.y = buf.z;
        buf.z = buf.w;
        avail--;
        return r;
    }
};

// Three Philox blocks with interleaved rounds (independent chains overlap).
__device__ __forceinline__ void philox4x32_10_x3(uint4& a, uint4& b, uint4& c, uint2 k) {
#pragma unroll
    for (int r = 0; r < 10; r++) {
        const uint32_t alo0 = 0xD2511F53u * a.x, ahi0 = __umulhi(0xD2511F53u, a.x);
        const uint32_t alo1 = 0xCD9E8D57u * a.z, ahi1 = __umulhi(0xCD9E8D57u, a.z);
        const uint32_t blo0 = 0xD2511F53u * b.x, bhi0 = __umulhi(0xD2511F53u, b.x);
        const uint32_t blo1 = 0xCD9E8D57u * b.z, bhi1 = __umulhi(0xCD9E8D57u, b.z);
        const uint32_t clo0 = 0xD2511F53u * c.x, chi0 = __umulhi(0xD2511F53u, c.x);
        const uint32_t clo1 = 0xCD9E8D57u * c.z, chi1 = __umulhi(0xCD9E8D57u, c.z);
        a = make_uint4(ahi1 ^ a.y ^ k.x, alo1, ahi0 ^ a.w ^ k.y, alo0);
        b = make_uint4(bhi1 ^ b.y ^ k.x, blo1, bhi0 ^ b.w ^ k.y, blo0);
        c = make_uint4(chi1 ^ c.y ^ k.x, clo1, chi0 ^ c.w ^ k.y, clo0);
        k.x += 0x9E3779B9u;
        k.y += 0xBB67AE85u;
    }
}

// A per-thread Philox stream buffered twelve words at a time; the sweep
// fills it before its first colour class so that no draw waits on a Philox
// chain inside a class.
struct ThreadRng12 {
    uint4 b0, b1, b2;
    uint32_t avail;
    uint32_t calls;
    uint4 ctr;   // (thread id, sweep lo, sweep hi, call index)
    uint2 key;

    // The first block of uniforms is generated at the first draw: a thread
    // whose moves are all downhill never runs Philox (the stream is the same).
    __device__ __forceinline__ void start(uint2 k, uint32_t tid, unsigned long long sweep, uint32_t call0 = 0u) {
        key = k;
        ctr = make_uint4(tid, (uint32_t)sweep, (uint32_t)(sweep >> 32), 0u);
        calls = call0;
        avail = 0;
    }
    __device__ __forceinline__ void refill() {
        uint4 a = ctr, b = ctr, c = ctr;
        a.w = calls;
        b.w = calls + 1;
        c.w = calls + 2;
        calls += 3;
        philox4x32_10_x3(a, b, c, key);
        b0 = a;
        b1 = b;
        b2 = c;
        avail = 12;
    }
    // The same stream one Philox block at a time, for threads that draw few
    // words per sweep (the twelve-word refill would compute eight unused);
    // a stream is drawn with next() or with next_one(), not both.
    __device__ __forceinline__ uint32_t next_one() {
        if (avail == 0) {
            uint4 a = ctr;
            a.w = calls++;
            b0 = philox4x32_10(a, key);
            avail = 4;
        }
        const uint32_t r = b0.x;
        b0 = make_uint4(b0.y, b0.z, b0.w, 0u);
        avail--;
        return r;
    }
    __device__ __forceinline__ uint32_t next() {
        if (avail == 0) refill();
        const uint32_t r = b0.x;
        b0 = make_uint4(b0.y, b0.z, b0.w, b1.x);
        b1 = make_uint4(b1.y, b1.z, b1.w, b2.x);
        b2 = make_uint4(b2.y, b2.z, b2.w, 0u);
        avail--;
        return r;
    }
};

// Uniform in (0, 1] from the top 24 bits (never zero, so log() is finite).
__device__ __forceinline__ float u01_open0(uint32_t x) {
    return ((float)(x >> 8) + 1.0f) * (1.0f / 16777216.0f);
}

// Integer in [0, range) by the high word of a 32x32 product (range < 2^32).
__device__ __forceinline__ uint32_t bounded32(uint32_t x, uint32_t range) {
    return __umulhi(x, range);
}

// ---------------------------------------------------- cross-block memory
__device__ __forceinline__ long long ld_cg(const long long* p) { return __ldcg(p); }
__device__ __forceinline__ int8_t ld_cg(const int8_t* p) { return (int8_t)__ldcg((const signed char*)p); }

// -------------------------------------------------------- group barrier
__device__ __forceinline__ unsigned int ld_acquire_gpu(const unsigned int* p) {
    unsigned int v;
    asm volatile("ld.acquire.gpu.global.u32 %0, [%1];" : "=r"(v) : "l"(p) : "memory");
    return v;
}

__device__ __forceinline__ unsigned int atom_add_acq_rel_gpu(unsigned int* p, unsigned int x) {
    unsigned int old;
    asm volatile("atom.acq_rel.gpu.global.add.u32 %0, [%1], %2;" : "=r"(old) : "l"(p), "r"(x) : "memory");
    return old;
}

__device__ __forceinline__ void red_add_release_gpu(unsigned int* p, unsigned int x) {
    asm volatile("red.release.gpu.global.add.u32 [%0], %1;" ::"l"(p), "r"(x) : "memory");
}

__device__ __forceinline__ unsigned long long ld_relaxed_gpu_u64(const unsigned long long* p) {
    unsigned long long v;
    asm volatile("ld.relaxed.gpu.global.u64 %0, [%1];" : "=l"(v) : "l"(p) : "memory");
    return v;
}

__device__ __forceinline__ void fence_acq_rel_gpu() {
    asm volatile("fence.acq_rel.gpu;" ::: "memory");
}

__device__ __forceinline__ void st_release_gpu_u64(unsigned long long* p, unsigned long long v) {
    asm volatile("st.release.gpu.global.u64 [%0], %1;" ::"l"(p), "l"(v) : "memory");
}

// A replica's published energy word: the publishing step's tag in the high
// half, the energy (it fits 32 bits: the launch checks the problem's energy
// range) in the low half.  Tags come from a counter that never repeats and
// never gives 0, so neither a zeroed word nor one left by an earlier step or
// launch matches the tag being waited for.
__device__ __forceinline__ unsigned long long pub_word(uint32_t tag, long long E) {
    return ((unsigned long long)tag << 32) | (unsigned long long)(uint32_t)(int32_t)E;
}

// A counting barrier over `nblocks` co-resident blocks (guaranteed by a
// cooperative launch).  Arrivals are counted in bar[0] with an acquire-
// release add (it publishes the block's writes, ordered before it by the
// block barrier, and acquires the earlier arrivers'); the last arriver
// resets the count and bumps the generation bar[1] with a release, which
// the others poll with acquire loads.  `gen` is thread 0's copy of the
// generation (read when the block joins the group; the generation cannot
// move before every block has arrived), so arriving costs one atomic.
// Waits are bounded: after `limit_ns`, or when another block has raised
// `abort`, the barrier records the failure and returns false.  Callers
// return when it fails.  `nblocks` may exceed the blocks that arrive (a
// test hook counts arrivals that never come, so that every wait runs out).
__device__ __forceinline__ bool group_barrier(unsigned int* bar, unsigned int nblocks, volatile int* abort_flag,
                                              DevStatus* st, unsigned int& gen,
                                              unsigned long long limit_ns = kWaitLimitNs) {
    __shared__ int s_ok;
    __syncthreads();
    if (threadIdx.x == 0) {
        const unsigned int g = gen;
        const unsigned int arrived = atom_add_acq_rel_gpu(bar, 1u);
        int ok = 1;
        if (arrived == nblocks - 1) {
            atomicExch(bar, 0u);
            red_add_release_gpu(bar + 1, 1u);
        } else {
            const unsigned long long t0 = globaltimer_ns();
            unsigned int spins = 0;
            while (ld_acquire_gpu(bar + 1) == g) {
                if (*abort_flag) { ok = 0; break; }
                if ((++spins & 63u) == 0 && globaltimer_ns() - t0 > limit_ns) {
                    dev_fail(st, abort_flag, DEV_BARRIER_TIMEOUT, 1, blockIdx.x, g);
                    ok = 0;
                    break;
                }
                __nanosleep(32);
            }
        }
        gen = g + 1u;
        s_ok = ok;
    }
    __syncthreads();
    return s_ok != 0;
}

// ------------------------------------------------- bulk-copy (TMA) staging
// One-dimensional cp.async.bulk global->shared copies completing on an
// mbarrier.  Addresses must be 16-byte aligned and sizes multiples of 16.
__device__ __forceinline__ uint32_t smem_u32(const void* p) {
    return (uint32_t)__cvta_generic_to_shared(p);
}

__device__ __forceinline__ void mbar_init(uint64_t* bar, uint32_t count) {
    asm volatile("mbarrier.init.shared::cta.b64 [%0], %1;" ::"r"(smem_u32(bar)), "r"(count) : "memory");
    asm volatile("fence.proxy.async.shared::cta;" ::: "memory");
}

__device__ __forceinline__ void mbar_expect_tx(uint64_t* bar, uint32_t bytes) {
    asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;" ::"r"(smem_u32(bar)), "r"(bytes)
                 : "memory");
}

__device__ __forceinline__ void bulk_g2s(void* dst, const void* src, uint32_t bytes, uint64_t* bar) {
    asm volatile(
        "cp.async.bulk.shared::cluster.global.mbarrier::complete_tx::bytes [%0], [%1], %2, [%3];" ::"r"(
            smem_u32(dst)),
        "l"(src), "r"(bytes), "r"(smem_u32(bar))
        : "memory");
}

__device__ __forceinline__ bool mbar_try_wait(uint64_t* bar, uint32_t parity) {
    uint32_t done;
    asm volatile(
        "{\n\t.reg .pred p;\n\t"
        "mbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\n\t"
        "selp.u32 %0, 1, 0, p;\n\t}"
        : "=r"(done)
        : "r"(smem_u32(bar)), "r"(parity)
        : "memory");
    return done != 0;
}

// Bounded wait for phase `parity` of an mbarrier; false on timeout.
__device__ __forceinline__ bool mbar_wait_bounded(uint64_t* bar, uint32_t parity,
                                                  unsigned long long limit_ns = kWaitLimitNs) {
    const unsigned long long t0 = globaltimer_ns();
    unsigned int spins = 0;
    while (!mbar_try_wait(bar, parity)) {
        if ((++spins & 255u) == 0 && globaltimer_ns() - t0 > limit_ns) return false;
    }
    return true;
}

}  // namespace pticm
