// mlp.cu -- the surrogate ln g(E) network: a 4 x 256 SiLU MLP whose forward
// and backward GEMMs run on the tcgen05 tensor cores (tc_gemm.cu), BF16
// operands with FP32 accumulation, trained with Adam on FP32 master weights.
#include <cuda_bf16.h>
#include <cuda_runtime.h>

#include <algorithm>
#include <cmath>
#include <cstring>
#include <string>
#include <vector>

#include "pticm.h"
#include "pticm_engine.h"
#include "runtime_internal.h"

namespace pticm {
cudaError_t tc_gemm(const __nv_bfloat16* A, const __nv_bfloat16* B, int M, int N, int K, const float* bias, int act,
                    float* Cf, __nv_bfloat16* Cb, long long ldc, DevStatus* status, int* abort_flag,
                    cudaStream_t st);
}  // namespace pticm

using namespace pticm;

namespace {

int mlp_fail(int code, const std::string& m) {
    set_last_error(m);
    return code;
}

#define MLP_CK(x)                                                                                         \
    do {                                                                                                  \
        cudaError_t e_ = (x);                                                                             \
        if (e_ != cudaSuccess) return mlp_fail(PTICM_ERR_CUDA, std::string(#x) + ": " + cudaGetErrorString(e_)); \
    } while (0)

}  // namespace

extern "C" int pticm_tc_gemm_check(int M, int N, int K, const uint16_t* A, const uint16_t* B, const float* bias,
                                   int act, float* C, uint16_t* C_bf16) {
    if (M <= 0 || N <= 0 || K <= 0 || (K % 64) || !A || !B || !C)
        return mlp_fail(PTICM_ERR_INVALID, "need positive M, N and K a multiple of 64");
    int count = 0;
    if (cudaGetDeviceCount(&count) != cudaSuccess || count == 0)
        return mlp_fail(PTICM_ERR_NODEVICE, "no CUDA device is available");
    __nv_bfloat16 *dA = nullptr, *dB = nullptr;
    float *dC = nullptr, *db = nullptr;
    __nv_bfloat16* dCb = nullptr;
    DevStatus* ds = nullptr;
    int* dab = nullptr;
    int rc = PTICM_OK;
    auto cleanup = [&]() {
        cudaFree(dA); cudaFree(dB); cudaFree(dC); cudaFree(dCb); cudaFree(db); cudaFree(ds); cudaFree(dab);
    };
    if (cudaMalloc(&dA, (size_t)M * K * 2) || cudaMalloc(&dB, (size_t)N * K * 2) ||
        cudaMalloc(&dC, (size_t)M * N * 4) || cudaMalloc(&ds, sizeof(DevStatus)) || cudaMalloc(&dab, 4) ||
        (bias && cudaMalloc(&db, (size_t)N * 4)) || (C_bf16 && cudaMalloc(&dCb, (size_t)M * N * 2))) {
        cleanup();
        return mlp_fail(PTICM_ERR_NOMEM, "device allocation failed");
    }
    cudaError_t e = cudaMemcpy(dA, A, (size_t)M * K * 2, cudaMemcpyHostToDevice);
    if (e == cudaSuccess) e = cudaMemcpy(dB, B, (size_t)N * K * 2, cudaMemcpyHostToDevice);
    if (e == cudaSuccess && bias) e = cudaMemcpy(db, bias, (size_t)N * 4, cudaMemcpyHostToDevice);
    if (e == cudaSuccess) e = cudaMemset(ds, 0, sizeof(DevStatus));
    if (e == cudaSuccess) e = cudaMemset(dab, 0, 4);
    if (e == cudaSuccess) e = tc_gemm(dA, dB, M, N, K, db, act, dC, dCb, N, ds, dab, nullptr);
    if (e == cudaSuccess) e = cudaDeviceSynchronize();
    DevStatus hs{};
    if (e == cudaSuccess) e = cudaMemcpy(&hs, ds, sizeof hs, cudaMemcpyDeviceToHost);
    if (e == cudaSuccess) e = cudaMemcpy(C, dC, (size_t)M * N * 4, cudaMemcpyDeviceToHost);
    if (e == cudaSuccess && C_bf16) e = cudaMemcpy(C_bf16, dCb, (size_t)M * N * 2, cudaMemcpyDeviceToHost);
    if (e != cudaSuccess) rc = mlp_fail(PTICM_ERR_CUDA, std::string("tc_gemm: ") + cudaGetErrorString(e));
    else if (hs.error) rc = mlp_fail(PTICM_ERR_DEVICE, "tc_gemm: tensor-core wait expired");
    cleanup();
    return rc;
}

extern "C" int pticm_tc_gemm_bench(int M, int N, int K, int iters, double* ms_per_gemm, double* tflops) {
    if (M <= 0 || N <= 0 || K <= 0 || (K % 64) || iters <= 0 || !ms_per_gemm)
        return mlp_fail(PTICM_ERR_INVALID, "need positive M, N, iters and K a multiple of 64");
    int count = 0;
    if (cudaGetDeviceCount(&count) != cudaSuccess || count == 0)
        return mlp_fail(PTICM_ERR_NODEVICE, "no CUDA device is available");
    __nv_bfloat16 *dA = nullptr, *dB = nullptr, *dC = nullptr;
    DevStatus* ds = nullptr;
    int* dab = nullptr;
    cudaEvent_t e0 = nullptr, e1 = nullptr;
    auto cleanup = [&]() {
        cudaFree(dA); cudaFree(dB); cudaFree(dC); cudaFree(ds); cudaFree(dab);
        if (e0) cudaEventDestroy(e0);
        if (e1) cudaEventDestroy(e1);
    };
    if (cudaMalloc(&dA, (size_t)M * K * 2) || cudaMalloc(&dB, (size_t)N * K * 2) || cudaMalloc(&dC, (size_t)M * N * 2) ||
        cudaMalloc(&ds, sizeof(DevStatus)) || cudaMalloc(&dab, 4)) {
        cleanup();
        return mlp_fail(PTICM_ERR_NOMEM, "device allocation failed");
    }
    cudaError_t e = cudaMemset(dA, 0x3c, (size_t)M * K * 2);   // bf16 ~1.0 everywhere: finite sums
    if (e == cudaSuccess) e = cudaMemset(dB, 0x3c, (size_t)N * K * 2);
    if (e == cudaSuccess) e = cudaMemset(ds, 0, sizeof(DevStatus));
    if (e == cudaSuccess) e = cudaMemset(dab, 0, 4);
    if (e == cudaSuccess) e = cudaEventCreate(&e0);
    if (e == cudaSuccess) e = cudaEventCreate(&e1);
    if (e == cudaSuccess) e = tc_gemm(dA, dB, M, N, K, nullptr, 0, nullptr, dC, N, ds, dab, nullptr);   // warm-up
    if (e == cudaSuccess) e = cudaEventRecord(e0, nullptr);
    for (int i = 0; i < iters && e == cudaSuccess; i++)
        e = tc_gemm(dA, dB, M, N, K, nullptr, 0, nullptr, dC, N, ds, dab, nullptr);
    if (e == cudaSuccess) e = cudaEventRecord(e1, nullptr);
    if (e == cudaSuccess) e = cudaEventSynchronize(e1);
    float ms = 0.f;
    if (e == cudaSuccess) e = cudaEventElapsedTime(&ms, e0, e1);
    DevStatus hs{};
    if (e == cudaSuccess) e = cudaMemcpy(&hs, ds, sizeof hs, cudaMemcpyDeviceToHost);
    int rc = PTICM_OK;
    if (e != cudaSuccess) rc = mlp_fail(PTICM_ERR_CUDA, std::string("tc_gemm: ") + cudaGetErrorString(e));
    else if (hs.error) rc = mlp_fail(PTICM_ERR_DEVICE, "tc_gemm: tensor-core wait expired");
    else {
        *ms_per_gemm = (double)ms / iters;
        if (tflops) *tflops = 2.0 * M * N * (double)K / (*ms_per_gemm * 1e-3) / 1e12;
    }
    cleanup();
    return rc;
}

// ===================================================================== MLP
namespace {

constexpr int MLP_IN = 7;         // features + normalised energy
constexpr int MLP_K0 = 64;        // input width padded for the GEMM
constexpr int MLP_H = 256;        // hidden width
constexpr int MLP_LAYERS = 4;     // hidden layers

// flat parameter layout: W1 [H x K0], b1, W2 [H x H], b2, W3, b3, W4, b4, w5 [H], b5
constexpr size_t kW1 = 0, kB1 = kW1 + (size_t)MLP_H * MLP_K0;
constexpr size_t kW2 = kB1 + MLP_H, kB2 = kW2 + (size_t)MLP_H * MLP_H;
constexpr size_t kW3 = kB2 + MLP_H, kB3 = kW3 + (size_t)MLP_H * MLP_H;
constexpr size_t kW4 = kB3 + MLP_H, kB4 = kW4 + (size_t)MLP_H * MLP_H;
constexpr size_t kW5 = kB4 + MLP_H, kB5 = kW5 + MLP_H;
constexpr size_t kParams = kB5 + 1;

const size_t kWoff[MLP_LAYERS] = {kW1, kW2, kW3, kW4};
const size_t kBoff[MLP_LAYERS] = {kB1, kB2, kB3, kB4};
const int kKin[MLP_LAYERS] = {MLP_K0, MLP_H, MLP_H, MLP_H};

__device__ __forceinline__ float silu_grad(float z) {
    const float s = 1.0f / (1.0f + __expf(-z));
    return s * (1.0f + z * (1.0f - s));
}

// inputs -> bf16 [B x 64] (columns >= 7 zero) and targets.  idx holds the
// batch's dataset rows (null: rows 0..n_valid-1); with `iter` set, idx is a
// ring of `ring` batches of n_valid rows and the batch is number *iter mod ring
__global__ void mlp_gather(const float* X, const float* Y, const uint32_t* idx, const long long* iter, int ring,
                           int B, int n_valid, __nv_bfloat16* X0, float* t) {
    const int b = blockIdx.x;
    const int c = threadIdx.x;   // 64 threads
    const bool valid = b < n_valid;
    if (iter) idx += (*iter % ring) * (long long)n_valid;
    const long long s = valid ? (long long)(idx ? idx[b] : (uint32_t)b) : 0;
    const float v = (valid && c < MLP_IN) ? X[s * MLP_IN + c] : 0.0f;
    X0[(long long)b * MLP_K0 + c] = __float2bfloat16_rn(v);
    if (c == 0) t[b] = valid ? Y[s] : 0.0f;
}

// y_b = H4_b . w5 + b5 ; loss (sum of squares) ; dy_b = 2 (y_b - t_b) / n
__global__ void mlp_out_fwd(const __nv_bfloat16* H4, const float* w5, const float* b5, const float* t, int n_valid,
                            float* y, float* dy, float* loss) {
    const int b = blockIdx.x * (blockDim.x >> 5) + (threadIdx.x >> 5);
    const int lane = threadIdx.x & 31;
    if (b >= gridDim.x * (blockDim.x >> 5)) return;
    float acc = 0.0f;
    for (int j = lane; j < MLP_H; j += 32) acc += __bfloat162float(H4[(long long)b * MLP_H + j]) * w5[j];
    for (int o = 16; o > 0; o >>= 1) acc += __shfl_xor_sync(0xffffffffu, acc, o);
    if (lane == 0) {
        const float v = acc + b5[0];
        y[b] = v;
        if (dy) {
            const bool valid = b < n_valid;
            const float e = valid ? v - t[b] : 0.0f;
            dy[b] = valid ? 2.0f * e / (float)n_valid : 0.0f;
            if (loss) atomicAdd(loss, e * e);
        }
    }
}

// dZ4 = dy w5 * silu'(Z4): fp32 and bf16 copies plus the bf16 transpose
__global__ void mlp_out_bwd(const float* dy, const float* w5, const float* Z4, int B, float* dZf, __nv_bfloat16* dZ,
                            __nv_bfloat16* dZT) {
    const long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x;
    if (i >= (long long)B * MLP_H) return;
    const int b = (int)(i / MLP_H), j = (int)(i % MLP_H);
    const float d = dy[b] * w5[j] * silu_grad(Z4[i]);
    dZf[i] = d;
    dZ[i] = __float2bfloat16_rn(d);
    dZT[(long long)j * B + b] = __float2bfloat16_rn(d);
}

// dZ = dH * silu'(Z)
__global__ void mlp_silu_bwd(const float* dH, const float* Z, int B, float* dZf, __nv_bfloat16* dZ,
                             __nv_bfloat16* dZT) {
    const long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x;
    if (i >= (long long)B * MLP_H) return;
    const int b = (int)(i / MLP_H), j = (int)(i % MLP_H);
    const float d = dH[i] * silu_grad(Z[i]);
    dZf[i] = d;
    dZ[i] = __float2bfloat16_rn(d);
    dZT[(long long)j * B + b] = __float2bfloat16_rn(d);
}

// out[c][r] = in[r][c] for a bf16 rows x cols matrix
__global__ void mlp_transpose(const __nv_bfloat16* in, int rows, int cols, __nv_bfloat16* out) {
    __shared__ __nv_bfloat16 tile[32][33];
    const int c0 = blockIdx.x * 32, r0 = blockIdx.y * 32;
    for (int k = threadIdx.y; k < 32; k += blockDim.y) {
        const int r = r0 + k, c = c0 + threadIdx.x;
        if (r < rows && c < cols) tile[k][threadIdx.x] = in[(long long)r * cols + c];
    }
    __syncthreads();
    for (int k = threadIdx.y; k < 32; k += blockDim.y) {
        const int c = c0 + k, r = r0 + threadIdx.x;
        if (r < rows && c < cols) out[(long long)c * rows + r] = tile[threadIdx.x][k];
    }
}

// Column sums over the batch in a fixed order (deterministic): a 32 x 32
// block covers 32 columns, thread row y sums batch rows y, y+32, ..., then
// row 0 adds the 32 partial sums.  Each column is read as 128-byte lines.
constexpr int kSumRows = 32;

// db[j] = sum_b dZ[b][j]  (fp32)
__global__ void mlp_colsum(const float* dZ, int B, int cols, float* db) {
    __shared__ float part[kSumRows][33];
    const int j = blockIdx.x * 32 + threadIdx.x;
    float s = 0.0f;
    if (j < cols)
        for (int b = threadIdx.y; b < B; b += kSumRows) s += dZ[(long long)b * cols + j];
    part[threadIdx.y][threadIdx.x] = s;
    __syncthreads();
    if (threadIdx.y == 0 && j < cols) {
        float t = 0.0f;
        for (int k = 0; k < kSumRows; k++) t += part[k][threadIdx.x];
        db[j] = t;
    }
}

// dw5[j] = sum_b dy_b H4[b][j] (blocks 0..7, as mlp_colsum); db5 = sum_b dy_b
// (the last block: thread (x, y) sums rows y*32+x + 1024 k, then a fixed tree)
__global__ void mlp_out_wgrad(const float* dy, const __nv_bfloat16* H4, int B, float* dw5, float* db5) {
    __shared__ float part[kSumRows][33];
    const bool bias = blockIdx.x == gridDim.x - 1;
    const int j = blockIdx.x * 32 + threadIdx.x;
    float s = 0.0f;
    if (bias) {
        for (int b = threadIdx.y * 32 + threadIdx.x; b < B; b += 32 * kSumRows) s += dy[b];
    } else {
        for (int b = threadIdx.y; b < B; b += kSumRows) s += dy[b] * __bfloat162float(H4[(long long)b * MLP_H + j]);
    }
    part[threadIdx.y][threadIdx.x] = s;
    __syncthreads();
    if (threadIdx.y != 0) return;
    float t = 0.0f;
    for (int k = 0; k < kSumRows; k++) t += part[k][threadIdx.x];
    if (!bias) {
        dw5[j] = t;
        return;
    }
    for (int o = 16; o > 0; o >>= 1) t += __shfl_xor_sync(0xffffffffu, t, o);
    if (threadIdx.x == 0) db5[0] = t;
}

// Adam (Kingma & Ba 2015) with bias correction on the flat parameters; the
// step number is the device counter *step + 1 (the counter moves in
// mlp_step_end, so a captured training step replays unchanged)
__global__ void mlp_adam(float* p, const float* g, float* m, float* v, long long n, float lr, float b1, float b2,
                         float eps, const long long* step) {
    const long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x;
    if (i >= n) return;
    const float k = (float)(*step + 1);
    const float c1 = 1.0f - powf(b1, k), c2 = 1.0f - powf(b2, k);
    const float gi = g[i];
    const float mi = b1 * m[i] + (1.0f - b1) * gi;
    const float vi = b2 * v[i] + (1.0f - b2) * gi * gi;
    m[i] = mi;
    v[i] = vi;
    p[i] -= lr * (mi / c1) / (sqrtf(vi / c2) + eps);
}

// bf16 copies of a weight matrix [rows x cols] and of its transpose
__global__ void mlp_weights_bf16(const float* W, int rows, int cols, __nv_bfloat16* Wb, __nv_bfloat16* WTb) {
    const long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x;
    if (i >= (long long)rows * cols) return;
    const int r = (int)(i / cols), c = (int)(i % cols);
    const __nv_bfloat16 x = __float2bfloat16_rn(W[i]);
    Wb[i] = x;
    WTb[(long long)c * rows + r] = x;
}

// end of a training step: the step's mean loss, then both counters advance
__global__ void mlp_step_end(const float* loss, float n_valid, long long* ctr, float* losses) {
    losses[ctr[0]] = *loss / n_valid;
    ctr[0]++;
    ctr[1]++;
}

}  // namespace

struct pticm_mlp {
    int B = 0;                        // batch capacity (multiple of 128)
    float* P = nullptr;               // fp32 master parameters
    float* G = nullptr;               // gradients
    float* Mm = nullptr;              // Adam first moments
    float* Vm = nullptr;              // Adam second moments
    __nv_bfloat16* Wb[MLP_LAYERS] = {};
    __nv_bfloat16* WTb[MLP_LAYERS] = {};
    __nv_bfloat16* X0 = nullptr;      // [B x 64]
    __nv_bfloat16* H[MLP_LAYERS] = {};   // [B x 256]
    float* Z[MLP_LAYERS] = {};        // [B x 256]
    __nv_bfloat16* HT[MLP_LAYERS] = {};  // transposes of X0, H1, H2, H3
    float* dZf = nullptr;
    __nv_bfloat16* dZ = nullptr;
    __nv_bfloat16* dZT = nullptr;
    float* dH = nullptr;              // [B x 256]
    float *t = nullptr, *y = nullptr, *dy = nullptr, *loss = nullptr;
    float *dX = nullptr, *dY = nullptr;   // dataset on the device
    uint32_t* idx = nullptr;
    size_t data_n = 0;
    long long* ctr = nullptr;         // device: [0] iteration of the current training call, [1] Adam steps taken
    DevStatus* status = nullptr;
    int* abort_flag = nullptr;
    std::vector<void*> allocs;
    ~pticm_mlp() {
        for (void* p : allocs) cudaFree(p);
    }
    template <typename T>
    cudaError_t alloc(T** p, size_t count) {
        void* q = nullptr;
        cudaError_t e = cudaMalloc(&q, count * sizeof(T));
        if (e != cudaSuccess) return e;
        allocs.push_back(q);
        *p = static_cast<T*>(q);
        return cudaMemset(q, 0, count * sizeof(T));
    }
};

namespace {

int mlp_refresh_bf16(pticm_mlp* m, cudaStream_t st) {
    for (int l = 0; l < MLP_LAYERS; l++) {
        const long long cnt = (long long)MLP_H * kKin[l];
        mlp_weights_bf16<<<(unsigned)((cnt + 255) / 256), 256, 0, st>>>(m->P + kWoff[l], MLP_H, kKin[l], m->Wb[l],
                                                                        m->WTb[l]);
    }
    MLP_CK(cudaGetLastError());
    return PTICM_OK;
}

int mlp_check_status(pticm_mlp* m) {
    DevStatus hs{};
    MLP_CK(cudaMemcpy(&hs, m->status, sizeof hs, cudaMemcpyDeviceToHost));
    if (hs.error) return mlp_fail(PTICM_ERR_DEVICE, "surrogate network: tensor-core wait expired");
    return PTICM_OK;
}

// forward for rows [0, n) of the staged batch; Z and H kept for backward
int mlp_forward(pticm_mlp* m, int n_valid, bool with_loss, cudaStream_t st) {
    const int B = m->B;
    const __nv_bfloat16* in = m->X0;
    for (int l = 0; l < MLP_LAYERS; l++) {
        MLP_CK(tc_gemm(in, m->Wb[l], B, MLP_H, kKin[l], m->P + kBoff[l], 1, m->Z[l], m->H[l], MLP_H, m->status,
                       m->abort_flag, st));
        in = m->H[l];
    }
    if (with_loss) MLP_CK(cudaMemsetAsync(m->loss, 0, sizeof(float), st));
    mlp_out_fwd<<<B / 8, 256, 0, st>>>(m->H[3], m->P + kW5, m->P + kB5, m->t, n_valid, m->y, with_loss ? m->dy : nullptr,
                                with_loss ? m->loss : nullptr);
    MLP_CK(cudaGetLastError());
    return PTICM_OK;
}

int mlp_backward(pticm_mlp* m, cudaStream_t st) {
    const int B = m->B;
    const dim3 tb(32, 8);
    // transposes of the layer inputs X0, H1, H2, H3
    const __nv_bfloat16* ins[MLP_LAYERS] = {m->X0, m->H[0], m->H[1], m->H[2]};
    for (int l = 0; l < MLP_LAYERS; l++)
        mlp_transpose<<<dim3((kKin[l] + 31) / 32, (B + 31) / 32), tb, 0, st>>>(ins[l], B, kKin[l], m->HT[l]);
    const dim3 sb(32, kSumRows);
    mlp_out_wgrad<<<MLP_H / 32 + 1, sb, 0, st>>>(m->dy, m->H[3], B, m->G + kW5, m->G + kB5);
    const long long elems = (long long)B * MLP_H;
    mlp_out_bwd<<<(unsigned)((elems + 255) / 256), 256, 0, st>>>(m->dy, m->P + kW5, m->Z[3], B, m->dZf, m->dZ, m->dZT);
    MLP_CK(cudaGetLastError());
    for (int l = MLP_LAYERS - 1; l >= 0; l--) {
        // dW_l = dZ_l^T . X_l  (M = 256 outputs, N = inputs, K = batch)
        MLP_CK(tc_gemm(m->dZT, m->HT[l], MLP_H, kKin[l], B, nullptr, 0, m->G + kWoff[l], nullptr, kKin[l], m->status,
                       m->abort_flag, st));
        mlp_colsum<<<MLP_H / 32, sb, 0, st>>>(m->dZf, B, MLP_H, m->G + kBoff[l]);
        if (l == 0) break;
        // dH_{l-1} = dZ_l . W_l  (B = W_l^T as [inputs x outputs])
        MLP_CK(tc_gemm(m->dZ, m->WTb[l], B, kKin[l], MLP_H, nullptr, 0, m->dH, nullptr, kKin[l], m->status,
                       m->abort_flag, st));
        mlp_silu_bwd<<<(unsigned)((elems + 255) / 256), 256, 0, st>>>(m->dH, m->Z[l - 1], B, m->dZf, m->dZ, m->dZT);
        MLP_CK(cudaGetLastError());
    }
    return PTICM_OK;
}

}  // namespace

extern "C" {

int pticm_mlp_create(uint64_t seed, uint32_t batch, pticm_mlp** out) {
    if (!out || batch == 0) return mlp_fail(PTICM_ERR_INVALID, "invalid arguments");
    int count = 0;
    if (cudaGetDeviceCount(&count) != cudaSuccess || count == 0)
        return mlp_fail(PTICM_ERR_NODEVICE, "no CUDA device is available");
    auto m = new pticm_mlp();
    m->B = (int)((batch + 127) / 128 * 128);
    const size_t B = (size_t)m->B;
    bool bad = false;
    bad |= m->alloc(&m->P, kParams) != cudaSuccess;
    bad |= m->alloc(&m->G, kParams) != cudaSuccess;
    bad |= m->alloc(&m->Mm, kParams) != cudaSuccess;
    bad |= m->alloc(&m->Vm, kParams) != cudaSuccess;
    for (int l = 0; l < MLP_LAYERS; l++) {
        bad |= m->alloc(&m->Wb[l], (size_t)MLP_H * kKin[l]) != cudaSuccess;
        bad |= m->alloc(&m->WTb[l], (size_t)MLP_H * kKin[l]) != cudaSuccess;
        bad |= m->alloc(&m->H[l], B * MLP_H) != cudaSuccess;
        bad |= m->alloc(&m->Z[l], B * MLP_H) != cudaSuccess;
        bad |= m->alloc(&m->HT[l], B * kKin[l]) != cudaSuccess;
    }
    bad |= m->alloc(&m->X0, B * MLP_K0) != cudaSuccess;
    bad |= m->alloc(&m->dZf, B * MLP_H) != cudaSuccess;
    bad |= m->alloc(&m->dZ, B * MLP_H) != cudaSuccess;
    bad |= m->alloc(&m->dZT, B * MLP_H) != cudaSuccess;
    bad |= m->alloc(&m->dH, B * MLP_H) != cudaSuccess;
    bad |= m->alloc(&m->t, B) != cudaSuccess;
    bad |= m->alloc(&m->y, B) != cudaSuccess;
    bad |= m->alloc(&m->dy, B) != cudaSuccess;
    bad |= m->alloc(&m->loss, 1) != cudaSuccess;
    bad |= m->alloc(&m->idx, B) != cudaSuccess;
    bad |= m->alloc(&m->status, 1) != cudaSuccess;
    bad |= m->alloc(&m->abort_flag, 1) != cudaSuccess;
    bad |= m->alloc(&m->ctr, 2) != cudaSuccess;
    if (bad) {
        delete m;
        return mlp_fail(PTICM_ERR_NOMEM, "device allocation failed");
    }
    // He-style initialisation from a host generator; unused input columns 0
    std::vector<float> p(kParams, 0.0f);
    uint64_t s = seed * 0x9E3779B97F4A7C15ull + 0x1234567ull;
    auto gauss = [&]() {
        // Box-Muller on two splitmix64 draws
        auto next = [&]() {
            uint64_t z = (s += 0x9E3779B97F4A7C15ull);
            z = (z ^ (z >> 30)) * 0xBF58476D1CE4E5B9ull;
            z = (z ^ (z >> 27)) * 0x94D049BB133111EBull;
            z ^= z >> 31;
            return ((z >> 11) + 0.5) * (1.0 / 9007199254740992.0);
        };
        const double u1 = next(), u2 = next();
        return (float)(std::sqrt(-2.0 * std::log(u1)) * std::cos(6.283185307179586 * u2));
    };
    for (int l = 0; l < MLP_LAYERS; l++) {
        const int fan_in = l == 0 ? MLP_IN : MLP_H;
        const float sc = std::sqrt(2.0f / fan_in);
        for (int r = 0; r < MLP_H; r++)
            for (int c = 0; c < kKin[l]; c++)
                p[kWoff[l] + (size_t)r * kKin[l] + c] = (l == 0 && c >= MLP_IN) ? 0.0f : sc * gauss();
    }
    for (int j = 0; j < MLP_H; j++) p[kW5 + j] = std::sqrt(1.0f / MLP_H) * gauss();
    if (cudaMemcpy(m->P, p.data(), kParams * 4, cudaMemcpyHostToDevice) != cudaSuccess || mlp_refresh_bf16(m, 0)) {
        delete m;
        return mlp_fail(PTICM_ERR_CUDA, "parameter upload failed");
    }
    *out = m;
    return PTICM_OK;
}

void pticm_mlp_destroy(pticm_mlp* m) { delete m; }

uint64_t pticm_mlp_param_count(void) { return kParams; }

int pticm_mlp_get_params(pticm_mlp* m, float* out) {
    if (!m || !out) return mlp_fail(PTICM_ERR_INVALID, "null argument");
    MLP_CK(cudaMemcpy(out, m->P, kParams * 4, cudaMemcpyDeviceToHost));
    return PTICM_OK;
}

int pticm_mlp_set_params(pticm_mlp* m, const float* in) {
    if (!m || !in) return mlp_fail(PTICM_ERR_INVALID, "null argument");
    MLP_CK(cudaMemcpy(m->P, in, kParams * 4, cudaMemcpyHostToDevice));
    return mlp_refresh_bf16(m, 0);
}

int pticm_mlp_set_data(pticm_mlp* m, const float* x, const float* y, uint64_t n) {
    if (!m || !x || !y || n == 0) return mlp_fail(PTICM_ERR_INVALID, "invalid arguments");
    if (m->dX) { cudaFree(m->dX); cudaFree(m->dY); }
    m->dX = m->dY = nullptr;
    MLP_CK(cudaMalloc(&m->dX, n * MLP_IN * 4));
    MLP_CK(cudaMalloc(&m->dY, n * 4));
    MLP_CK(cudaMemcpy(m->dX, x, n * MLP_IN * 4, cudaMemcpyHostToDevice));
    MLP_CK(cudaMemcpy(m->dY, y, n * 4, cudaMemcpyHostToDevice));
    m->data_n = n;
    return PTICM_OK;
}

int pticm_mlp_gradients(pticm_mlp* m, const float* x, const float* y, uint32_t n, float* grads, float* loss) {
    if (!m || !x || !y || n == 0 || (int)n > m->B) return mlp_fail(PTICM_ERR_INVALID, "invalid arguments");
    if (int rc = pticm_mlp_set_data(m, x, y, n)) return rc;
    MLP_CK(cudaMemset(m->status, 0, sizeof(DevStatus)));
    mlp_gather<<<m->B, MLP_K0>>>(m->dX, m->dY, nullptr, nullptr, 1, m->B, (int)n, m->X0, m->t);
    MLP_CK(cudaGetLastError());
    if (int rc = mlp_forward(m, (int)n, true, 0)) return rc;
    if (int rc = mlp_backward(m, 0)) return rc;
    MLP_CK(cudaDeviceSynchronize());
    if (int rc = mlp_check_status(m)) return rc;
    if (grads) MLP_CK(cudaMemcpy(grads, m->G, kParams * 4, cudaMemcpyDeviceToHost));
    if (loss) {
        float l = 0;
        MLP_CK(cudaMemcpy(&l, m->loss, 4, cudaMemcpyDeviceToHost));
        *loss = l / (float)n;
    }
    return PTICM_OK;
}

int pticm_mlp_train(pticm_mlp* m, const float* x, const float* y, uint64_t n, uint32_t steps, float lr,
                    uint64_t seed, float* loss_per_step) {
    if (!m || !x || !y || n == 0 || n > 0xFFFFFFFFull) return mlp_fail(PTICM_ERR_INVALID, "invalid arguments");
    if (int rc = pticm_mlp_set_data(m, x, y, n)) return rc;
    if (steps == 0) return PTICM_OK;
    const int B = m->B;
    const int nb = (int)std::min<uint64_t>(n, (uint64_t)B);
    // Batches: an epoch-wise Fisher-Yates shuffle on the host (xorshift64),
    // written a chunk of kChunk steps at a time into one half of a pinned
    // two-chunk ring; the device ring (the same layout) is read by the
    // captured step at row (iteration mod 2 kChunk).  The host fills chunk
    // c + 2 while chunk c + 1 runs.
    constexpr uint32_t kChunk = 256;
    const size_t half = (size_t)kChunk * nb;
    std::vector<uint32_t> order(n);
    for (uint64_t i = 0; i < n; i++) order[i] = (uint32_t)i;
    uint64_t s = seed ^ 0xA0761D6478BD642Full;
    auto nxt = [&]() {
        s ^= s << 13; s ^= s >> 7; s ^= s << 17;
        return s;
    };
    uint64_t cursor = n;
    auto fill = [&](uint32_t* dst, uint32_t count) {
        for (size_t k = 0; k < (size_t)count * nb; k++) {
            if (cursor == n) {   // reshuffle each epoch
                for (uint64_t i = n - 1; i > 0; i--) std::swap(order[i], order[nxt() % (i + 1)]);
                cursor = 0;
            }
            dst[k] = order[cursor++];
        }
    };

    struct Res {
        cudaStream_t st = nullptr;
        cudaGraph_t graph = nullptr;
        cudaGraphExec_t exec = nullptr;
        uint32_t* ring = nullptr;    // device, 2 kChunk batches
        uint32_t* hring = nullptr;   // pinned host
        float* losses = nullptr;     // device, one per step
        cudaEvent_t copied[2] = {nullptr, nullptr};
        ~Res() {
            if (st) cudaStreamSynchronize(st);
            if (exec) cudaGraphExecDestroy(exec);
            if (graph) cudaGraphDestroy(graph);
            for (cudaEvent_t e : copied)
                if (e) cudaEventDestroy(e);
            if (st) cudaStreamDestroy(st);
            cudaFree(ring);
            cudaFree(losses);
            cudaFreeHost(hring);
        }
    } r;
    MLP_CK(cudaStreamCreateWithFlags(&r.st, cudaStreamNonBlocking));
    MLP_CK(cudaMalloc(&r.ring, 2 * half * 4));
    MLP_CK(cudaMalloc(&r.losses, (size_t)steps * 4));
    MLP_CK(cudaMallocHost(&r.hring, 2 * half * 4));
    for (cudaEvent_t& e : r.copied) MLP_CK(cudaEventCreateWithFlags(&e, cudaEventDisableTiming));
    MLP_CK(cudaMemsetAsync(m->status, 0, sizeof(DevStatus), r.st));
    MLP_CK(cudaMemsetAsync(m->ctr, 0, sizeof(long long), r.st));   // this call's iteration counter

    // one training step, captured once: gather, forward with loss, backward,
    // Adam, bf16 weight copies, counters (37 kernels and one memset)
    MLP_CK(cudaStreamBeginCapture(r.st, cudaStreamCaptureModeRelaxed));
    int rc = PTICM_OK;
    mlp_gather<<<B, MLP_K0, 0, r.st>>>(m->dX, m->dY, r.ring, m->ctr, 2 * (int)kChunk, B, nb, m->X0, m->t);
    if (!rc) rc = mlp_forward(m, nb, true, r.st);
    if (!rc) rc = mlp_backward(m, r.st);
    if (!rc) {
        mlp_adam<<<(unsigned)((kParams + 255) / 256), 256, 0, r.st>>>(m->P, m->G, m->Mm, m->Vm, (long long)kParams,
                                                                       lr, 0.9f, 0.999f, 1e-8f, m->ctr + 1);
        rc = mlp_refresh_bf16(m, r.st);
    }
    if (!rc) mlp_step_end<<<1, 1, 0, r.st>>>(m->loss, (float)nb, m->ctr, r.losses);
    const cudaError_t ec = cudaStreamEndCapture(r.st, &r.graph);
    if (rc) return rc;
    MLP_CK(ec);
    MLP_CK(cudaGraphInstantiate(&r.exec, r.graph, 0));

    for (uint32_t c0 = 0, chunk = 0; c0 < steps; c0 += kChunk, chunk++) {
        const uint32_t cnt = std::min(kChunk, steps - c0);
        const int h = (int)(chunk & 1);
        // the pinned half is free once its previous upload (two chunks ago) ran
        MLP_CK(cudaEventSynchronize(r.copied[h]));
        fill(r.hring + h * half, cnt);
        MLP_CK(cudaMemcpyAsync(r.ring + h * half, r.hring + h * half, (size_t)cnt * nb * 4, cudaMemcpyHostToDevice,
                               r.st));
        MLP_CK(cudaEventRecord(r.copied[h], r.st));
        for (uint32_t i = 0; i < cnt; i++) MLP_CK(cudaGraphLaunch(r.exec, r.st));
    }
    if (loss_per_step)
        MLP_CK(cudaMemcpyAsync(loss_per_step, r.losses, (size_t)steps * 4, cudaMemcpyDeviceToHost, r.st));
    MLP_CK(cudaStreamSynchronize(r.st));
    return mlp_check_status(m);
}

int pticm_mlp_predict(pticm_mlp* m, const float* x, uint64_t n, float* y) {
    if (!m || !x || !y) return mlp_fail(PTICM_ERR_INVALID, "null argument");
    if (n == 0) return PTICM_OK;
    std::vector<float> zeros(n, 0.0f);
    if (int rc = pticm_mlp_set_data(m, x, zeros.data(), n)) return rc;
    MLP_CK(cudaMemset(m->status, 0, sizeof(DevStatus)));
    const int B = m->B;
    std::vector<uint32_t> batch(B);
    for (uint64_t base = 0; base < n; base += (uint64_t)B) {
        const int nb = (int)std::min<uint64_t>((uint64_t)B, n - base);
        for (int b = 0; b < nb; b++) batch[b] = (uint32_t)(base + b);
        MLP_CK(cudaMemcpy(m->idx, batch.data(), (size_t)nb * 4, cudaMemcpyHostToDevice));
        mlp_gather<<<B, MLP_K0>>>(m->dX, m->dY, m->idx, nullptr, 1, B, nb, m->X0, m->t);
        if (int rc = mlp_forward(m, nb, false, 0)) return rc;
        MLP_CK(cudaMemcpy(y + base, m->y, (size_t)nb * 4, cudaMemcpyDeviceToHost));
    }
    return mlp_check_status(m);
}

}  // extern "C"
