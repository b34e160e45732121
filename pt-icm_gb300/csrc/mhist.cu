// mhist.cu -- FP64 multihistogram density of states on the GPU.
//
// The fixed point of src/cae_estimator.cc:172-253 (Ferrenberg-Swendsen /
// Newman-Barkema multihistogram): for energy bins e_i = emin + i*estep,
//   ln g(e_i) = ln sum_j N_j(e_i) - ln sum_j exp(ln n - ln Z_j - beta_j e_i)
//   ln Z_j    = ln sum_i exp(ln g(e_i) - beta_j e_i)
// iterated from ln Z = 0 until sum_j ((lnZ_j - lnZ'_j)/lnZ'_j)^2 <= tol.
// The reference accumulates every sum with a pairwise log-add in index order;
// here each log-sum-exp is a max-shifted sum of exponentials (one exp per
// term), the numerator is the exact integer count sum, and the bin sums are
// reduced in parallel -- the same quantities to FP64 rounding.  FP64 is kept
// throughout: the exponents span thousands of nats.
#include <cuda_runtime.h>

#include <algorithm>
#include <cfloat>
#include <cmath>
#include <cstdint>

namespace pticm {

constexpr int kMhistThreads = 256;

// ln g over all bins; one thread per bin, loops over the nt histograms.
__global__ void mh_bins_kernel(const uint32_t* hist, const uint64_t* hoff, const uint64_t* hlen,
                               const double* emin, const double* beta, const double* logZ, int nt, double estep,
                               double min_emin, double logn, long long nbins, double* logdos) {
    extern __shared__ double sm[];
    double* sZ = sm;
    double* sB = sm + nt;
    double* sE = sm + 2 * nt;
    for (int j = threadIdx.x; j < nt; j += blockDim.x) {
        sZ[j] = logZ[j];
        sB[j] = beta[j];
        sE[j] = emin[j];
    }
    __syncthreads();
    for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < nbins; i += (long long)gridDim.x * blockDim.x) {
        const double e = min_emin + (double)i * estep;
        double m = -DBL_MAX;
        unsigned long long count = 0;
        for (int j = 0; j < nt; j++) {
            m = fmax(m, logn - sZ[j] - sB[j] * e);
            if (e < sE[j]) continue;
            const double idx = floor((e - sE[j]) / estep);
            if (idx >= (double)hlen[j]) continue;
            count += hist[hoff[j] + (uint64_t)idx];
        }
        if (count == 0) {
            logdos[i] = -DBL_MAX;
            continue;
        }
        double s = 0.0;
        for (int j = 0; j < nt; j++) s += exp(logn - sZ[j] - sB[j] * e - m);
        logdos[i] = log((double)count) - (m + log(s));
    }
}

// Partial log-sum-exp of ln g(e_i) - beta_j e_i over one chunk of bins:
// block (chunk, j) writes its max and the shifted sum.
__global__ void mh_partials_kernel(const double* logdos, long long nbins, const double* beta, double estep,
                                   double min_emin, double* pmax, double* psum, int chunks) {
    const int j = blockIdx.y, c = blockIdx.x;
    const long long per = (nbins + chunks - 1) / chunks;
    const long long i0 = (long long)c * per, i1 = min(nbins, i0 + per);
    const double bj = beta[j];
    __shared__ double red[kMhistThreads / 32];
    double m = -DBL_MAX;
    for (long long i = i0 + threadIdx.x; i < i1; i += blockDim.x) m = fmax(m, logdos[i] - bj * ((double)i * estep + min_emin));
    for (int o = 16; o > 0; o >>= 1) m = fmax(m, __shfl_xor_sync(0xffffffffu, m, o));
    if ((threadIdx.x & 31) == 0) red[threadIdx.x >> 5] = m;
    __syncthreads();
    m = -DBL_MAX;
    for (int w = 0; w < (int)(blockDim.x >> 5); w++) m = fmax(m, red[w]);
    __syncthreads();
    double s = 0.0;
    for (long long i = i0 + threadIdx.x; i < i1; i += blockDim.x) s += exp(logdos[i] - bj * ((double)i * estep + min_emin) - m);
    for (int o = 16; o > 0; o >>= 1) s += __shfl_xor_sync(0xffffffffu, s, o);
    if ((threadIdx.x & 31) == 0) red[threadIdx.x >> 5] = s;
    __syncthreads();
    if (threadIdx.x == 0) {
        double t = 0.0;
        for (int w = 0; w < (int)(blockDim.x >> 5); w++) t += red[w];
        pmax[(size_t)j * chunks + c] = m;
        psum[(size_t)j * chunks + c] = t;
    }
}

// Combine the chunks per histogram, update ln Z and the convergence sum
// (accumulated in histogram order, as src/cae_estimator.cc:245-251 does).
__global__ void mh_finish_kernel(const double* pmax, const double* psum, int chunks, int nt, double* logZ,
                                 double* metric) {
    extern __shared__ double sd[];
    for (int j = threadIdx.x; j < nt; j += blockDim.x) {
        double M = -DBL_MAX;
        for (int c = 0; c < chunks; c++) M = fmax(M, pmax[(size_t)j * chunks + c]);
        double S = 0.0;
        for (int c = 0; c < chunks; c++) S += psum[(size_t)j * chunks + c] * exp(pmax[(size_t)j * chunks + c] - M);
        const double tz = M + log(S);
        const double q = fabs(logZ[j] - tz) / fabs(tz);
        sd[j] = q * q;
        logZ[j] = tz;
    }
    __syncthreads();
    if (threadIdx.x == 0) {
        double t = 0.0;
        for (int j = 0; j < nt; j++) t += sd[j];
        *metric = t;
    }
}

cudaError_t mhist_iterate(const uint32_t* hist, const uint64_t* hoff, const uint64_t* hlen, const double* emin,
                          const double* beta, double* logZ, int nt, double estep, double min_emin, double logn,
                          long long nbins, double* logdos, double* pmax, double* psum, int chunks, double* metric,
                          cudaStream_t st) {
    const int blocks = (int)std::min<long long>(4096, (nbins + kMhistThreads - 1) / kMhistThreads);
    mh_bins_kernel<<<blocks > 0 ? blocks : 1, kMhistThreads, 3 * nt * sizeof(double), st>>>(
        hist, hoff, hlen, emin, beta, logZ, nt, estep, min_emin, logn, nbins, logdos);
    mh_partials_kernel<<<dim3(chunks, nt), kMhistThreads, 0, st>>>(logdos, nbins, beta, estep, min_emin, pmax, psum,
                                                                   chunks);
    mh_finish_kernel<<<1, 1024, nt * sizeof(double), st>>>(pmax, psum, chunks, nt, logZ, metric);
    return cudaGetLastError();
}

}  // namespace pticm
