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
#include <cfloat>
#include <cstdint>

#include "mhist_job.h"

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

// ------------------------------------------------------------------------
// Whole fixed point on the device, one CTA per instance (many instances per
// launch).  Per iteration:
//   bins:  ln g_i = ln c_i - (m + ln sum_j exp(a_j - beta_j e_i - m)),
//          a_j = ln n - ln Z_j, c_i the summed counts of bin i;
//   temps: ln Z_j = m_j + ln sum_i exp(ln g_i - beta_j e_i - m_j)   (one warp per j)
// until sum_j ((lnZ_j - lnZ'_j)/lnZ'_j)^2 <= 1e-7 (or the iteration cap).
// The shifts m, m_j and the test that drops a term come from FP32 shadows
// of the same quantities; every kept term and every sum is FP64.  A term more
// than 60 nats below the shift is dropped: 60 nats is 1e-26 relative, so
// even 10^7 such terms stay below half an ulp of a sum that is >= 1 and the
// FP64 result is the one that keeps them.
namespace {
constexpr float kDropNats = 60.f;
}

__global__ void __launch_bounds__(256) mh_solve_kernel(const MhJob* jobs, const uint32_t* hist, const uint64_t* hoff,
                                                       const uint64_t* hlen, const double* emin, const double* beta,
                                                       double* logdos, double* logc, float* ldf, double* logZ,
                                                       unsigned long long* iters, long long max_iters) {
    const MhJob J = jobs[blockIdx.x];
    const int nt = J.nt, tid = threadIdx.x, T = blockDim.x, lane = tid & 31, warp = tid >> 5, nw = T >> 5;
    const long long nb = J.nbins;
    extern __shared__ double mh_sm[];
    double* sZ = mh_sm;            // nt
    double* sA = sZ + nt;          // nt: ln n - ln Z_j
    double* sB = sA + nt;          // nt
    double* sNew = sB + nt;        // nt
    float* sAf = reinterpret_cast<float*>(sNew + nt);
    float* sBf = sAf + nt;
    __shared__ int s_done;
    const uint64_t* ho = hoff + J.row0;
    const uint64_t* hl = hlen + J.row0;
    const double* em = emin + J.row0;
    double* ld = logdos + J.bin0;
    double* lc = logc + J.bin0;
    float* lf = ldf + J.bin0;
    for (int j = tid; j < nt; j += T) {
        sZ[j] = 0.0;
        sB[j] = beta[J.row0 + j];
        sBf[j] = (float)sB[j];
    }
    // summed counts per bin (constant over the iterations)
    for (long long i = tid; i < nb; i += T) {
        const double e = J.min_emin + (double)i * J.estep;
        unsigned long long count = 0;
        for (int j = 0; j < nt; j++) {
            if (e < em[j]) continue;
            const double idx = floor((e - em[j]) / J.estep);
            if (idx >= (double)hl[j]) continue;
            count += hist[ho[j] + (uint64_t)idx];
        }
        lc[i] = count ? log((double)count) : -DBL_MAX;
    }
    __syncthreads();
    long long it = 0;
    for (; it < max_iters; it++) {
        for (int j = tid; j < nt; j += T) {
            sA[j] = J.logn - sZ[j];
            sAf[j] = (float)sA[j];
        }
        __syncthreads();
        // bins
        for (long long i = tid; i < nb; i += T) {
            const double lci = lc[i];
            if (lci == -DBL_MAX) {
                ld[i] = -DBL_MAX;
                lf[i] = -FLT_MAX;
                continue;
            }
            const double e = J.min_emin + (double)i * J.estep;
            const float ef = (float)e;
            float mf = -FLT_MAX;
            for (int j = 0; j < nt; j++) mf = fmaxf(mf, sAf[j] - sBf[j] * ef);
            const double m = (double)mf;
            double s = 0.0;
            for (int j = 0; j < nt; j++) {
                if (sAf[j] - sBf[j] * ef - mf < -kDropNats) continue;
                s += exp(sA[j] - sB[j] * e - m);
            }
            const double v = lci - (m + log(s));
            ld[i] = v;
            lf[i] = (float)v;
        }
        __syncthreads();
        // temperatures: one warp per ln Z_j
        for (int j = warp; j < nt; j += nw) {
            const float bf = sBf[j];
            const double bj = sB[j];
            float mf = -FLT_MAX;
            for (long long i = lane; i < nb; i += 32) {
                const float v = lf[i];
                if (v == -FLT_MAX) continue;
                mf = fmaxf(mf, v - bf * (float)(J.min_emin + (double)i * J.estep));
            }
            for (int o = 16; o > 0; o >>= 1) mf = fmaxf(mf, __shfl_xor_sync(0xffffffffu, mf, o));
            const double m = (double)mf;
            double s = 0.0;
            for (long long i = lane; i < nb; i += 32) {
                const float v = lf[i];
                if (v == -FLT_MAX) continue;
                const double e = J.min_emin + (double)i * J.estep;
                if (v - bf * (float)e - mf < -kDropNats) continue;
                s += exp(ld[i] - bj * e - m);
            }
            for (int o = 16; o > 0; o >>= 1) s += __shfl_xor_sync(0xffffffffu, s, o);
            if (lane == 0) sNew[j] = m + log(s);
        }
        __syncthreads();
        if (tid == 0) {
            double metric = 0.0;
            for (int j = 0; j < nt; j++) {
                const double q = fabs(sZ[j] - sNew[j]) / fabs(sNew[j]);
                metric += q * q;
                sZ[j] = sNew[j];
            }
            s_done = !(metric > 1e-7);
        }
        __syncthreads();
        if (s_done) { it++; break; }
    }
    for (int j = tid; j < nt; j += T) logZ[J.row0 + j] = sZ[j];
    if (tid == 0) iters[blockIdx.x] = (unsigned long long)it;
}

cudaError_t mhist_solve(const MhJob* jobs, int njobs, int max_nt, const uint32_t* hist, const uint64_t* hoff,
                        const uint64_t* hlen, const double* emin, const double* beta, double* logdos, double* logc,
                        float* ldf, double* logZ, unsigned long long* iters, long long max_iters, cudaStream_t st) {
    const size_t smem = (size_t)max_nt * (4 * sizeof(double) + 2 * sizeof(float));
    mh_solve_kernel<<<njobs, 256, smem, st>>>(jobs, hist, hoff, hlen, emin, beta, logdos, logc, ldf, logZ, iters,
                                              max_iters);
    return cudaGetLastError();
}

}  // namespace pticm
