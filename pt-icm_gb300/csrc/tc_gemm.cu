// tc_gemm.cu -- BF16 GEMM on the 5th-generation tensor cores (tcgen05, sm_103a)
// for the surrogate-ladder MLP.
//
//   C[M x N] = act(A[M x K] . B[N x K]^T + bias[N])      (A, B bf16, K-major)
//
// Two kernels compute the same 128 x BN tiles.  tc_gemm_tma_kernel (below)
// brings the operands in with the tensor memory accelerator; the kernel here
// is its fallback when the CUDA driver's tensor-map encoder is not available.
// One CTA of 128 threads computes a 128 x BN tile (BN = 128, or 256 when
// N > 128).  K advances in chunks of 64 through TC_STAGES (2 or 3) shared-
// memory buffers in the canonical K-major layout without swizzle: 8-row x 16-byte
// core matrices, K-adjacent core matrices 128 B apart (leading byte offset),
// 8-row groups 1024 B apart (stride byte offset).  The threads fill the
// buffers with 16-byte cp.async copies, TC_STAGES - 1 chunks ahead of the
// tensor cores.  Thread 0 issues tcgen05.mma.kind::f16 (M=128, N=BN, K=16
// each, FP32 accumulation) into a tensor-memory accumulator and commits each
// chunk to its buffer's mbarrier, which the threads wait on before they
// refill that buffer.  The four warps then read their 32 accumulator lanes
// with tcgen05.ld and apply the epilogue (bias, optional SiLU, FP32 and/or
// BF16 stores, 16 bytes at a time when aligned).  Every wait is bounded; a
// timeout is recorded in a status word.
#include <cuda.h>   // CUtensorMap and its enums (the encoder is fetched at run time)
#include <cuda_bf16.h>
#include <cuda_runtime.h>

#include <cstdint>

#include "pticm_device.cuh"

namespace pticm {

constexpr int TC_BM = 128, TC_BK = 64;
constexpr uint32_t TC_TMEM_COLS = 256;                   // FP32 accumulator columns (N <= 256)

enum TcAct : int { TC_ACT_NONE = 0, TC_ACT_SILU = 1 };

// Shared-memory matrix descriptor: start address, leading (K) and stride
// (M/N) byte offsets in 16-byte units, descriptor version 1, no swizzle.
__device__ __forceinline__ uint64_t tc_smem_desc(uint32_t saddr, uint32_t lbo, uint32_t sbo) {
    uint64_t d = 0;
    d |= (uint64_t)((saddr >> 4) & 0x3FFFu);
    d |= (uint64_t)((lbo >> 4) & 0x3FFFu) << 16;
    d |= (uint64_t)((sbo >> 4) & 0x3FFFu) << 32;
    d |= (uint64_t)1 << 46;
    return d;
}

// Instruction descriptor of kind::f16: FP32 accumulator, BF16 A and B, both
// K-major, N >> 3 at bit 17, M >> 4 at bit 24.
__host__ __device__ constexpr uint32_t tc_idesc_bf16(int M, int N) {
    return (1u << 4) | (1u << 7) | (1u << 10) | ((uint32_t)(N >> 3) << 17) | ((uint32_t)(M >> 4) << 24);
}

__device__ __forceinline__ void tc_fence_proxy_async() {
    asm volatile("fence.proxy.async.shared::cta;" ::: "memory");
}


// Epilogue of one accumulator row segment: 32 FP32 columns from cb on,
// plus bias, stored as FP32 (pre-activation) and/or BF16 (after the
// optional SiLU); 16-byte stores when the row is aligned and complete.
__device__ __forceinline__ void tc_store_row(const uint32_t (&r)[32], int row, int cb, int N,
                                             const float* __restrict__ bias, int act, float* __restrict__ Cf,
                                             __nv_bfloat16* __restrict__ Cb, long long ldc, bool vec) {
    if (cb + 32 <= N && vec) {
        float v[32];
#pragma unroll
        for (int j = 0; j < 32; j++) v[j] = __uint_as_float(r[j]) + (bias ? __ldg(bias + cb + j) : 0.0f);
        if (Cf) {
            float4* o = reinterpret_cast<float4*>(Cf + (long long)row * ldc + cb);
#pragma unroll
            for (int q = 0; q < 8; q++) o[q] = make_float4(v[4 * q], v[4 * q + 1], v[4 * q + 2], v[4 * q + 3]);
        }
        if (act == TC_ACT_SILU)
#pragma unroll
            for (int j = 0; j < 32; j++) v[j] = v[j] / (1.0f + __expf(-v[j]));
        if (Cb) {
            uint4* o = reinterpret_cast<uint4*>(Cb + (long long)row * ldc + cb);
#pragma unroll
            for (int q = 0; q < 4; q++) {
                uint32_t w4[4];
#pragma unroll
                for (int h = 0; h < 4; h++) {
                    const __nv_bfloat162 t = __floats2bfloat162_rn(v[8 * q + 2 * h], v[8 * q + 2 * h + 1]);
                    w4[h] = *reinterpret_cast<const uint32_t*>(&t);
                }
                o[q] = make_uint4(w4[0], w4[1], w4[2], w4[3]);
            }
        }
    } else {
#pragma unroll
        for (int j = 0; j < 32; j++) {
            const int col = cb + j;
            if (col >= N) continue;
            float v = __uint_as_float(r[j]) + (bias ? bias[col] : 0.0f);
            if (Cf) Cf[(long long)row * ldc + col] = v;
            if (act == TC_ACT_SILU) v = v / (1.0f + __expf(-v));
            if (Cb) Cb[(long long)row * ldc + col] = __float2bfloat16_rn(v);
        }
    }
}

__device__ __forceinline__ void cp_async16(uint32_t dst, const void* src, uint32_t src_bytes) {
    asm volatile("cp.async.cg.shared.global [%0], [%1], 16, %2;" ::"r"(dst), "l"(src), "r"(src_bytes) : "memory");
}
__device__ __forceinline__ void cp_async_commit() { asm volatile("cp.async.commit_group;" ::: "memory"); }
template <int N>
__device__ __forceinline__ void cp_async_wait() { asm volatile("cp.async.wait_group %0;" ::"n"(N) : "memory"); }

// Issue the copies of a tile of `nrows` x 64 bf16 (rows r0.., columns k0..)
// of a K-major matrix into the core-matrix layout (8-row x 16-byte core
// matrices, K-adjacent ones 128 B apart, 8-row groups 1024 B apart).  Lane
// pairs of 16-byte pieces cover a row's 128 bytes; rows past `rows` are
// zero-filled (no bytes read).
__device__ __forceinline__ void tc_stage_tile_async(uint8_t* dst, const __nv_bfloat16* src, long long ld, int r0,
                                                    int k0, int rows, int nrows) {
    const uint32_t d0 = smem_u32(dst);
    for (int idx = threadIdx.x; idx < nrows * 8; idx += blockDim.x) {
        const int m = idx >> 3, c = idx & 7;
        const bool in = r0 + m < rows;
        const __nv_bfloat16* p = in ? src + (long long)(r0 + m) * ld + k0 + c * 8 : src;
        cp_async16(d0 + (uint32_t)((m >> 3) * 1024 + (m & 7) * 16 + c * 128), p, in ? 16u : 0u);
    }
}

// One CTA computes a 128 x BN tile.  Chunk kc lives in buffer kc % TC_STAGES;
// after the MMAs of chunk kc are issued, the buffer of chunk kc - 1 is
// refilled with chunk kc + TC_STAGES - 1 once the commit of chunk kc - 1 has
// arrived (each mbarrier has at most one phase outstanding).  One cp.async
// group is committed per iteration, so waiting until TC_STAGES - 2 groups
// are pending means chunk kc + 1 has landed.
template <int BN, int TC_STAGES>
__global__ void __launch_bounds__(128, 1)
tc_gemm_kernel(const __nv_bfloat16* __restrict__ A, const __nv_bfloat16* __restrict__ B, int M, int N, int K,
               const float* __restrict__ bias, int act, float* __restrict__ Cf, __nv_bfloat16* __restrict__ Cb,
               long long ldc, DevStatus* status, int* abort_flag) {
    constexpr uint32_t A_BYTES = TC_BM * TC_BK * 2;
    constexpr uint32_t STAGE = A_BYTES + BN * TC_BK * 2;
    extern __shared__ __align__(1024) uint8_t tc_smem[];
    __shared__ uint64_t mbar[TC_STAGES];
    __shared__ uint32_t tmem_base_s;
    const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
    const int m0 = blockIdx.x * TC_BM, n0 = blockIdx.y * BN;
    uint8_t* buf0 = tc_smem;

    if (warp == 0) {
        asm volatile("tcgen05.alloc.cta_group::1.sync.aligned.shared::cta.b32 [%0], %1;" ::"r"(smem_u32(&tmem_base_s)),
                     "r"(TC_TMEM_COLS)
                     : "memory");
        asm volatile("tcgen05.relinquish_alloc_permit.cta_group::1.sync.aligned;" ::: "memory");
    }
    if (threadIdx.x == 0)
        for (int b = 0; b < TC_STAGES; b++) mbar_init(&mbar[b], 1);
    asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory");
    __syncthreads();
    asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
    const uint32_t tmem = tmem_base_s;
    const uint32_t idesc = tc_idesc_bf16(TC_BM, BN);
    const int nk = K / TC_BK;
    uint32_t ph[TC_STAGES];
    for (int b = 0; b < TC_STAGES; b++) ph[b] = 0u;

    // prologue: chunks 0 .. TC_STAGES-2, one group each (empty past nk)
    for (int c = 0; c < TC_STAGES - 1; c++) {
        if (c < nk) {
            uint8_t* dst = buf0 + c * STAGE;
            tc_stage_tile_async(dst, A, K, m0, c * TC_BK, M, TC_BM);
            tc_stage_tile_async(dst + A_BYTES, B, K, n0, c * TC_BK, N, BN);
        }
        cp_async_commit();
    }
    bool ok = true;
    for (int kc = 0; kc < nk; kc++) {
        const int b = kc % TC_STAGES;
        // chunk kc has landed: at most TC_STAGES-2 later groups are pending
        cp_async_wait<TC_STAGES - 2>();
        tc_fence_proxy_async();
        __syncthreads();
        if (threadIdx.x == 0) {
            asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
            const uint32_t aaddr = smem_u32(buf0 + b * STAGE), baddr = aaddr + A_BYTES;
#pragma unroll
            for (int kk = 0; kk < TC_BK / 16; kk++) {
                const uint64_t da = tc_smem_desc(aaddr + kk * 256, 128, 1024);
                const uint64_t db = tc_smem_desc(baddr + kk * 256, 128, 1024);
                const uint32_t accumulate = (kc > 0 || kk > 0) ? 1u : 0u;
                asm volatile(
                    "{\n\t.reg .pred p;\n\t"
                    "setp.ne.b32 p, %4, 0;\n\t"
                    "tcgen05.mma.cta_group::1.kind::f16 [%0], %1, %2, %3, p;\n\t}" ::"r"(tmem),
                    "l"(da), "l"(db), "r"(idesc), "r"(accumulate)
                    : "memory");
            }
            asm volatile("tcgen05.commit.cta_group::1.mbarrier::arrive::one.shared::cluster.b64 [%0];" ::"r"(
                             smem_u32(&mbar[b]))
                         : "memory");
        }
        // refill the buffer of chunk kc-1 with chunk kc+TC_STAGES-1
        const int nc = kc + TC_STAGES - 1;
        bool w = true;
        if (nc < nk) {
            const int rb = nc % TC_STAGES;
            if (kc >= 1) {   // that buffer was read by the MMAs of chunk kc-1
                w = mbar_wait_bounded(&mbar[rb], ph[rb]);
                ph[rb] ^= 1u;
            }
            if (w) {
                uint8_t* dst = buf0 + rb * STAGE;
                tc_stage_tile_async(dst, A, K, m0, nc * TC_BK, M, TC_BM);
                tc_stage_tile_async(dst + A_BYTES, B, K, n0, nc * TC_BK, N, BN);
            }
        }
        cp_async_commit();
        ok = __syncthreads_and(w) != 0;
        if (!ok) break;
    }
    cp_async_wait<0>();
    // drain: the last commit arrives when every MMA issued before it is done
    if (ok) {
        const int bl = (nk - 1) % TC_STAGES;
        ok = mbar_wait_bounded(&mbar[bl], ph[bl]);
    }
    ok = __syncthreads_and(ok) != 0;
    if (!ok) {
        // record the failure; give the MMAs in flight one more bounded wait
        // before the accumulator is released
        if (threadIdx.x == 0 && status) dev_fail(status, abort_flag, DEV_TMA_TIMEOUT, 100, blockIdx.x, blockIdx.y);
        mbar_wait_bounded(&mbar[(nk - 1) % TC_STAGES], ph[(nk - 1) % TC_STAGES]);
    }
    asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");

    // epilogue: warp w owns accumulator lanes (rows) 32w .. 32w+31; a row's
    // 32 columns go out as 16-byte stores when the output rows are aligned
    const int row = m0 + warp * 32 + lane;
    const bool vec_f = Cf == nullptr || (((reinterpret_cast<uintptr_t>(Cf) & 15) == 0) && (ldc & 3) == 0);
    const bool vec_b = Cb == nullptr || (((reinterpret_cast<uintptr_t>(Cb) & 15) == 0) && (ldc & 7) == 0);
    if (ok) {
#pragma unroll 1
        for (int c0 = 0; c0 < BN; c0 += 32) {
            uint32_t r[32];
            const uint32_t taddr = tmem + ((uint32_t)(warp * 32) << 16) + (uint32_t)c0;
            asm volatile(
                "tcgen05.ld.sync.aligned.32x32b.x32.b32 {%0,%1,%2,%3,%4,%5,%6,%7,%8,%9,%10,%11,%12,%13,%14,%15,"
                "%16,%17,%18,%19,%20,%21,%22,%23,%24,%25,%26,%27,%28,%29,%30,%31}, [%32];"
                : "=r"(r[0]), "=r"(r[1]), "=r"(r[2]), "=r"(r[3]), "=r"(r[4]), "=r"(r[5]), "=r"(r[6]), "=r"(r[7]),
                  "=r"(r[8]), "=r"(r[9]), "=r"(r[10]), "=r"(r[11]), "=r"(r[12]), "=r"(r[13]), "=r"(r[14]),
                  "=r"(r[15]), "=r"(r[16]), "=r"(r[17]), "=r"(r[18]), "=r"(r[19]), "=r"(r[20]), "=r"(r[21]),
                  "=r"(r[22]), "=r"(r[23]), "=r"(r[24]), "=r"(r[25]), "=r"(r[26]), "=r"(r[27]), "=r"(r[28]),
                  "=r"(r[29]), "=r"(r[30]), "=r"(r[31])
                : "r"(taddr));
            asm volatile("tcgen05.wait::ld.sync.aligned;" ::: "memory");
            if (row >= M) continue;
            tc_store_row(r, row, n0 + c0, N, bias, act, Cf, Cb, ldc, vec_f && vec_b);
        }
    }
    asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory");
    __syncthreads();
    if (warp == 0)
        asm volatile("tcgen05.dealloc.cta_group::1.sync.aligned.b32 %0, %1;" ::"r"(tmem), "r"(TC_TMEM_COLS) : "memory");
}

// ------------------------------------------------------------ TMA variant
// The same tile, with the operands brought in by the tensor memory
// accelerator: thread 0 issues cp.async.bulk.tensor loads of 64-wide K
// chunks (128 bytes a row) in the 128-byte swizzle, four stages ahead, each
// completing on its stage's "full" mbarrier; it issues the MMAs of a chunk
// when that barrier completes and commits them to the stage's "empty"
// mbarrier, which it waits on before loading the stage again.  The shared-
// memory descriptors use the matching SWIZZLE_128B K-major layout: 8-row x
// 128-byte atoms 1024 bytes apart, each K=16 step 32 bytes further into the
// atom.  Stage buffers start on 1024 bytes.
constexpr int TC_TMA_STAGES = 4;

__device__ __forceinline__ uint64_t tc_smem_desc_sw128(uint32_t saddr) {
    uint64_t d = 0;
    d |= (uint64_t)((saddr >> 4) & 0x3FFFu);
    d |= (uint64_t)1 << 16;              // leading byte offset (unused for swizzled K-major)
    d |= (uint64_t)(1024 >> 4) << 32;    // stride byte offset: 8-row atoms 1024 B apart
    d |= (uint64_t)1 << 46;              // descriptor version
    d |= (uint64_t)2 << 61;              // SWIZZLE_128B
    return d;
}

__device__ __forceinline__ void tma_load_2d(uint32_t dst, const CUtensorMap* map, int x, int y, uint64_t* bar) {
    asm volatile(
        "cp.async.bulk.tensor.2d.shared::cluster.global.mbarrier::complete_tx::bytes [%0], [%1, {%2, %3}], [%4];" ::"r"(
            dst),
        "l"(reinterpret_cast<uint64_t>(map)), "r"(x), "r"(y), "r"(smem_u32(bar))
        : "memory");
}

template <int BN>
__global__ void __launch_bounds__(128, 1)
tc_gemm_tma_kernel(const __grid_constant__ CUtensorMap mapA, const __grid_constant__ CUtensorMap mapB, int M, int N,
                   int K, const float* __restrict__ bias, int act, float* __restrict__ Cf,
                   __nv_bfloat16* __restrict__ Cb, long long ldc, DevStatus* status, int* abort_flag) {
    constexpr int S = TC_TMA_STAGES;
    constexpr uint32_t A_BYTES = TC_BM * TC_BK * 2;
    constexpr uint32_t STAGE = A_BYTES + BN * TC_BK * 2;
    extern __shared__ __align__(1024) uint8_t tc_smem[];
    __shared__ uint64_t full[S], empty[S];
    __shared__ uint32_t tmem_base_s;
    __shared__ int ok_s;
    const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
    const int m0 = blockIdx.x * TC_BM, n0 = blockIdx.y * BN;
    // stage buffers on 1024 bytes (the swizzle atom); the launch adds 1 KB
    const uint32_t base = (smem_u32(tc_smem) + 1023u) & ~1023u;

    if (warp == 0) {
        asm volatile("tcgen05.alloc.cta_group::1.sync.aligned.shared::cta.b32 [%0], %1;" ::"r"(smem_u32(&tmem_base_s)),
                     "r"(TC_TMEM_COLS)
                     : "memory");
        asm volatile("tcgen05.relinquish_alloc_permit.cta_group::1.sync.aligned;" ::: "memory");
    }
    if (threadIdx.x == 0) {
        for (int b = 0; b < S; b++) {
            mbar_init(&full[b], 1);
            mbar_init(&empty[b], 1);
        }
        ok_s = 1;
    }
    asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory");
    __syncthreads();
    asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
    const uint32_t tmem = tmem_base_s;
    const int nk = K / TC_BK;

    if (threadIdx.x == 0) {
        const uint32_t idesc = tc_idesc_bf16(TC_BM, BN);
        uint32_t pf[S], pe[S];
        for (int b = 0; b < S; b++) pf[b] = pe[b] = 0u;
        int issued = 0, consumed = 0;
        auto issue = [&](int c) {
            const int b = c % S;
            const uint32_t a_dst = base + (uint32_t)b * STAGE;
            mbar_expect_tx(&full[b], STAGE);
            tma_load_2d(a_dst, &mapA, c * TC_BK, m0, &full[b]);
            tma_load_2d(a_dst + A_BYTES, &mapB, c * TC_BK, n0, &full[b]);
        };
        bool ok = true;
        for (; issued < S && issued < nk; issued++) issue(issued);
        for (int kc = 0; kc < nk && ok; kc++) {
            const int b = kc % S;
            ok = mbar_wait_bounded(&full[b], pf[b]);
            pf[b] ^= 1u;
            if (!ok) break;
            consumed = kc + 1;
            asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
            const uint32_t aaddr = base + (uint32_t)b * STAGE, baddr = aaddr + A_BYTES;
#pragma unroll
            for (int kk = 0; kk < TC_BK / 16; kk++) {
                const uint64_t da = tc_smem_desc_sw128(aaddr + kk * 32);
                const uint64_t db = tc_smem_desc_sw128(baddr + kk * 32);
                const uint32_t accumulate = (kc > 0 || kk > 0) ? 1u : 0u;
                asm volatile(
                    "{\n\t.reg .pred p;\n\t"
                    "setp.ne.b32 p, %4, 0;\n\t"
                    "tcgen05.mma.cta_group::1.kind::f16 [%0], %1, %2, %3, p;\n\t}" ::"r"(tmem),
                    "l"(da), "l"(db), "r"(idesc), "r"(accumulate)
                    : "memory");
            }
            asm volatile("tcgen05.commit.cta_group::1.mbarrier::arrive::one.shared::cluster.b64 [%0];" ::"r"(
                             smem_u32(&empty[b]))
                         : "memory");
            if (issued < nk) {
                // the stage is free once this chunk's MMAs are done
                ok = mbar_wait_bounded(&empty[b], pe[b]);
                pe[b] ^= 1u;
                if (!ok) break;
                issue(issued++);
            }
        }
        if (ok) {
            // the last commit arrives when every MMA issued before it is done
            const int bl = (nk - 1) % S;
            ok = mbar_wait_bounded(&empty[bl], pe[bl]);
        }
        if (!ok) {
            if (status) dev_fail(status, abort_flag, DEV_TMA_TIMEOUT, 101, blockIdx.x, blockIdx.y);
            // the copies still in flight land before the CTA leaves (bounded)
            for (int c = consumed; c < issued; c++) {
                const int b = c % S;
                mbar_wait_bounded(&full[b], pf[b]);
                pf[b] ^= 1u;
            }
            mbar_wait_bounded(&empty[(nk - 1) % S], pe[(nk - 1) % S]);
            ok_s = 0;
        }
    }
    __syncthreads();
    asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
    const bool ok = ok_s != 0;

    // epilogue (as tc_gemm_kernel)
    const int row = m0 + warp * 32 + lane;
    const bool vec_f = Cf == nullptr || (((reinterpret_cast<uintptr_t>(Cf) & 15) == 0) && (ldc & 3) == 0);
    const bool vec_b = Cb == nullptr || (((reinterpret_cast<uintptr_t>(Cb) & 15) == 0) && (ldc & 7) == 0);
    if (ok) {
#pragma unroll 1
        for (int c0 = 0; c0 < BN; c0 += 32) {
            uint32_t r[32];
            const uint32_t taddr = tmem + ((uint32_t)(warp * 32) << 16) + (uint32_t)c0;
            asm volatile(
                "tcgen05.ld.sync.aligned.32x32b.x32.b32 {%0,%1,%2,%3,%4,%5,%6,%7,%8,%9,%10,%11,%12,%13,%14,%15,"
                "%16,%17,%18,%19,%20,%21,%22,%23,%24,%25,%26,%27,%28,%29,%30,%31}, [%32];"
                : "=r"(r[0]), "=r"(r[1]), "=r"(r[2]), "=r"(r[3]), "=r"(r[4]), "=r"(r[5]), "=r"(r[6]), "=r"(r[7]),
                  "=r"(r[8]), "=r"(r[9]), "=r"(r[10]), "=r"(r[11]), "=r"(r[12]), "=r"(r[13]), "=r"(r[14]),
                  "=r"(r[15]), "=r"(r[16]), "=r"(r[17]), "=r"(r[18]), "=r"(r[19]), "=r"(r[20]), "=r"(r[21]),
                  "=r"(r[22]), "=r"(r[23]), "=r"(r[24]), "=r"(r[25]), "=r"(r[26]), "=r"(r[27]), "=r"(r[28]),
                  "=r"(r[29]), "=r"(r[30]), "=r"(r[31])
                : "r"(taddr));
            asm volatile("tcgen05.wait::ld.sync.aligned;" ::: "memory");
            if (row >= M) continue;
            tc_store_row(r, row, n0 + c0, N, bias, act, Cf, Cb, ldc, vec_f && vec_b);
        }
    }
    asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory");
    __syncthreads();
    if (warp == 0)
        asm volatile("tcgen05.dealloc.cta_group::1.sync.aligned.b32 %0, %1;" ::"r"(tmem), "r"(TC_TMEM_COLS) : "memory");
}

template <int BN, int STAGES>
static cudaError_t tc_launch(const __nv_bfloat16* A, const __nv_bfloat16* B, int M, int N, int K, const float* bias,
                             int act, float* Cf, __nv_bfloat16* Cb, long long ldc, DevStatus* status,
                             int* abort_flag, cudaStream_t st) {
    const size_t smem = STAGES * (size_t)(TC_BM * TC_BK * 2 + BN * TC_BK * 2) + 1024;
    cudaError_t e =
        cudaFuncSetAttribute(tc_gemm_kernel<BN, STAGES>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
    if (e != cudaSuccess) return e;
    dim3 grid((M + TC_BM - 1) / TC_BM, (N + BN - 1) / BN);
    tc_gemm_kernel<BN, STAGES><<<grid, 128, smem, st>>>(A, B, M, N, K, bias, act, Cf, Cb, ldc, status, abort_flag);
    return cudaGetLastError();
}

// The CUDA driver's tensor-map encoder, fetched once through the runtime (no
// link against the driver library).
typedef CUresult (*EncodeTiledFn)(CUtensorMap*, CUtensorMapDataType, cuuint32_t, void*, const cuuint64_t*,
                                  const cuuint64_t*, const cuuint32_t*, const cuuint32_t*, CUtensorMapInterleave,
                                  CUtensorMapSwizzle, CUtensorMapL2promotion, CUtensorMapFloatOOBfill);

static EncodeTiledFn encode_tiled() {
    static const EncodeTiledFn fn = []() -> EncodeTiledFn {
        void* p = nullptr;
        cudaDriverEntryPointQueryResult q{};
        if (cudaGetDriverEntryPointByVersion("cuTensorMapEncodeTiled", &p, 12000, cudaEnableDefault, &q) !=
                cudaSuccess ||
            q != cudaDriverEntryPointSuccess)
            return nullptr;
        return reinterpret_cast<EncodeTiledFn>(p);
    }();
    return fn;
}

// A K-major bf16 matrix of `rows` x K as a 2-D tensor map: boxes of 64 x
// box_rows in the 128-byte swizzle, zeros outside the matrix.
static bool tc_tensor_map(CUtensorMap* map, const void* base, int rows, int K, int box_rows) {
    const EncodeTiledFn fn = encode_tiled();
    if (!fn) return false;
    const cuuint64_t dims[2] = {(cuuint64_t)K, (cuuint64_t)rows};
    const cuuint64_t strides[1] = {(cuuint64_t)K * 2};
    const cuuint32_t box[2] = {(cuuint32_t)TC_BK, (cuuint32_t)box_rows};
    const cuuint32_t elem[2] = {1, 1};
    return fn(map, CU_TENSOR_MAP_DATA_TYPE_BFLOAT16, 2, const_cast<void*>(base), dims, strides, box, elem,
              CU_TENSOR_MAP_INTERLEAVE_NONE, CU_TENSOR_MAP_SWIZZLE_128B, CU_TENSOR_MAP_L2_PROMOTION_L2_256B,
              CU_TENSOR_MAP_FLOAT_OOB_FILL_NONE) == CUDA_SUCCESS;
}

template <int BN>
static cudaError_t tc_launch_tma(const CUtensorMap& mapA, const CUtensorMap& mapB, int M, int N, int K,
                                 const float* bias, int act, float* Cf, __nv_bfloat16* Cb, long long ldc,
                                 DevStatus* status, int* abort_flag, cudaStream_t st) {
    const size_t smem = TC_TMA_STAGES * (size_t)(TC_BM * TC_BK * 2 + BN * TC_BK * 2) + 1024;
    cudaError_t e = cudaFuncSetAttribute(tc_gemm_tma_kernel<BN>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
    if (e != cudaSuccess) return e;
    dim3 grid((M + TC_BM - 1) / TC_BM, (N + BN - 1) / BN);
    tc_gemm_tma_kernel<BN><<<grid, 128, smem, st>>>(mapA, mapB, M, N, K, bias, act, Cf, Cb, ldc, status, abort_flag);
    return cudaGetLastError();
}

// Launch: M, N multiples of 128 not required (rows/cols beyond are masked),
// K a multiple of 64 and both operands 16-byte aligned with row stride K.
// N > 128 uses 128 x 256 tiles (one CTA covers a 256-wide layer).
cudaError_t tc_gemm(const __nv_bfloat16* A, const __nv_bfloat16* B, int M, int N, int K, const float* bias, int act,
                    float* Cf, __nv_bfloat16* Cb, long long ldc, DevStatus* status, int* abort_flag,
                    cudaStream_t st) {
    if (M <= 0 || N <= 0 || K < TC_BK || K % TC_BK != 0 ||
        ((reinterpret_cast<uintptr_t>(A) | reinterpret_cast<uintptr_t>(B)) & 15))
        return cudaErrorInvalidValue;
    // operands through the tensor memory accelerator when the CUDA driver's
    // tensor-map encoder is available (the row stride K*2 is a multiple of
    // 16 bytes and both bases 16-byte aligned, as TMA requires)
    {
        const int bn = N > 128 ? 256 : 128;
        CUtensorMap mapA, mapB;
        if (tc_tensor_map(&mapA, A, M, K, TC_BM) && tc_tensor_map(&mapB, B, N, K, bn)) {
            if (bn == 256)
                return tc_launch_tma<256>(mapA, mapB, M, N, K, bias, act, Cf, Cb, ldc, status, abort_flag, st);
            return tc_launch_tma<128>(mapA, mapB, M, N, K, bias, act, Cf, Cb, ldc, status, abort_flag, st);
        }
    }
    // (without the encoder: the threads copy the operands)
    // stage counts that leave room for two CTAs per SM (97 KB each): one
    // CTA's epilogue overlaps the other's loads (8192^3: 366 TFLOP/s against
    // 331 with four stages and one CTA)
    if (N > 128) return tc_launch<256, 2>(A, B, M, N, K, bias, act, Cf, Cb, ldc, status, abort_flag, st);
    return tc_launch<128, 3>(A, B, M, N, K, bias, act, Cf, Cb, ldc, status, abort_flag, st);
}

}  // namespace pticm
