// smem_rate.cu -- measured shared-memory copy rate of the GPU, the peak the
// engine's roofline is set against: the replicas and the staged adjacency of
// the single-instance and batched workloads live in shared memory, so the
// sweep's algorithmic bytes are shared-memory bytes.
//
// One block per SM, 1024 threads, copies a 96 KB region of its shared memory
// into another 96 KB region and back, 16 bytes per thread per access; the
// rate counts the bytes read plus the bytes written, as the HBM copy rate
// does.
#include <cuda_runtime.h>

#include <string>

#include "pticm.h"
#include "runtime_internal.h"

namespace {

constexpr int kRegionBytes = 96 * 1024;
constexpr int kThreads = 1024;

__global__ void __launch_bounds__(kThreads, 1) smem_copy_kernel(int iters, unsigned* sink) {
    extern __shared__ __align__(16) uint4 sm[];
    constexpr int per = kRegionBytes / 16;   // uint4 per region
    uint4* a = sm;
    uint4* b = sm + per;
    for (int i = threadIdx.x; i < per; i += blockDim.x) a[i] = make_uint4(i, i ^ 1, i ^ 2, i ^ 3);
    __syncthreads();
    for (int it = 0; it < iters; it++) {
        uint4* src = (it & 1) ? b : a;
        uint4* dst = (it & 1) ? a : b;
#pragma unroll
        for (int k = 0; k < per / kThreads; k++) {
            const int i = threadIdx.x + k * kThreads;
            uint4 v = src[i];
            v.x += 1u;
            dst[i] = v;
        }
        __syncthreads();
    }
    if (threadIdx.x == 0) atomicAdd(sink, a[blockIdx.x % per].x + b[0].y);
}

int sfail(int code, const std::string& m) {
    pticm::set_last_error(m);
    return code;
}

}  // namespace

extern "C" int pticm_smem_copy_rate(int iters, double* gb_per_s) {
    if (iters <= 0 || !gb_per_s) return sfail(PTICM_ERR_INVALID, "need iters > 0 and an output");
    int dev = 0, sms = 0, count = 0;
    if (cudaGetDeviceCount(&count) != cudaSuccess || count == 0)
        return sfail(PTICM_ERR_NODEVICE, "no CUDA device is available");
    if (cudaGetDevice(&dev) != cudaSuccess || cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev))
        return sfail(PTICM_ERR_CUDA, "device query failed");
    const int smem = 2 * kRegionBytes;
    cudaError_t e = cudaFuncSetAttribute(smem_copy_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, smem);
    pticm::DArr<unsigned> sink;
    if (e == cudaSuccess) e = sink.alloc(1);
    cudaEvent_t e0 = nullptr, e1 = nullptr;
    if (e == cudaSuccess) e = cudaEventCreate(&e0);
    if (e == cudaSuccess) e = cudaEventCreate(&e1);
    float ms = 0.f;
    if (e == cudaSuccess) {
        smem_copy_kernel<<<sms, kThreads, smem>>>(4, sink.p);   // warm-up
        cudaEventRecord(e0);
        smem_copy_kernel<<<sms, kThreads, smem>>>(iters, sink.p);
        cudaEventRecord(e1);
        e = cudaEventSynchronize(e1);
    }
    if (e == cudaSuccess) e = cudaGetLastError();
    if (e == cudaSuccess) e = cudaEventElapsedTime(&ms, e0, e1);
    if (e0) cudaEventDestroy(e0);
    if (e1) cudaEventDestroy(e1);
    if (e != cudaSuccess) return sfail(PTICM_ERR_CUDA, std::string("smem copy rate: ") + cudaGetErrorString(e));
    const double bytes = (double)sms * (double)iters * 2.0 * kRegionBytes;
    *gb_per_s = bytes / (ms * 1e-3) / 1e9;
    return PTICM_OK;
}
