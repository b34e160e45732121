// mhist_host.cc -- host side of the multihistogram ladder: the constant
// acceptance ("CAE") temperature walk of src/cae_estimator.cc:367-425.
//
// The walk itself is control flow on a handful of scalars and stays on the
// host in FP64.  Its cost is the pair acceptance of src/cae_estimator.cc:
// 262-293, a double sum over energy bins (O(nbins^2) log-adds in the
// reference).  With p1, p2 the log energy distributions at beta1 > beta2 and
// d = beta1 - beta2, it splits into
//   r = sum_i exp(p1_i) [ sum_{j<=i} exp(p2_j) + e^{d e_i} sum_{j>i} exp(p2_j - d e_j) ],
// a prefix and a suffix log-sum-exp: O(nbins) per candidate temperature.
#include <algorithm>
#include <cfloat>
#include <cmath>
#include <vector>

#include "mhist_host.h"

namespace pticm {

namespace {

inline double lse2(double a, double b) {   // log(e^a + e^b), a and b may be -inf
    if (a < b) std::swap(a, b);
    if (b == -INFINITY) return a;
    return a + std::log1p(std::exp(b - a));
}

}  // namespace

double partition_func(const std::vector<double>& logdos, double beta, double emin, double estep) {
    const size_t nb = logdos.size();
    double m = -DBL_MAX;
    for (size_t i = 0; i < nb; i++) m = std::max(m, logdos[i] - beta * ((double)i * estep + emin));
    double s = 0.0;
    for (size_t i = 0; i < nb; i++) s += std::exp(logdos[i] - beta * ((double)i * estep + emin) - m);
    return m + std::log(s);
}

static void pe_vec(const std::vector<double>& logdos, std::vector<double>& out, double emin, double beta, double logz,
                   double estep) {
    double e = emin;
    for (size_t i = 0; i < logdos.size(); i++, e += estep) out[i] = logdos[i] - e * beta - logz;
}

double acceptance_rate(const std::vector<double>& p1, const std::vector<double>& p2, double beta1, double beta2,
                       double estep, double emin) {
    const size_t nb = p1.size();
    if (nb == 0) return 0.0;
    const double d = beta1 - beta2;
    std::vector<double> suffix(nb + 1, -INFINITY);   // suffix[i] = log sum_{j>=i} exp(p2_j - d e_j)
    for (size_t j = nb; j-- > 0;) {
        const double ej = emin + (double)j * estep;
        suffix[j] = lse2(suffix[j + 1], p2[j] - d * ej);
    }
    double prefix = -INFINITY, total = -INFINITY;
    for (size_t i = 0; i < nb; i++) {
        prefix = lse2(prefix, p2[i]);
        const double ei = emin + (double)i * estep;
        const double inner = lse2(prefix, d * ei + suffix[i + 1]);
        total = lse2(total, p1[i] + inner);
    }
    return std::exp(total);
}

uint32_t cae_walk(const std::vector<double>& logdos, double min_emin, double estep, double beta_start,
                  double beta_end, double step_size, double r, uint32_t num_temps, double* bv) {
    const size_t nb = logdos.size();
    bv[0] = beta_start;
    double partition_last = partition_func(logdos, beta_start, min_emin, estep);
    double step = step_size;
    std::vector<double> prev(nb), curr(nb);
    pe_vec(logdos, prev, min_emin, beta_start, partition_last, estep);
    uint32_t i;
    for (i = 1; i < num_temps; i++) {
        const double beta_prev = bv[i - 1];
        bv[i] = beta_prev;
        double partition_curr = 0, r_curr = 0, r_last = -1;
        for (int guard = 0; guard < 100000; guard++) {
            bool cont = false;
            const double beta_orig = bv[i];
            bv[i] = 1 / (1 / bv[i] + step);
            partition_curr = partition_func(logdos, bv[i], min_emin, estep);
            pe_vec(logdos, curr, min_emin, bv[i], partition_curr, estep);
            r_curr = acceptance_rate(prev, curr, beta_prev, bv[i], estep, min_emin);
            if ((r - r_curr) > 0.05) {          // overshot: halve the step, retry from beta_orig
                bv[i] = beta_orig;
                step /= 2;
                cont = true;
            } else if (r_last > 0 && std::fabs(r_curr - r_last) < 5e-2) {
                step *= 2;                       // acceptance barely moves: take larger steps
            } else {
                r_last = r_curr;
            }
            if (!((r_curr > r && bv[i] > beta_end) || cont)) break;
        }
        if (bv[i] <= beta_end) break;
        partition_last = partition_curr;
        prev.swap(curr);
    }
    return i;
}

}  // namespace pticm
