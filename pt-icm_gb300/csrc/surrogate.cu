// surrogate.cu -- temperature ladders from the surrogate ln g(E) network
// (pticm_surrogate_*, pticm_learned_ladder, include/pticm.h).
//
// The network maps six instance features and the normalised energy
// x = E / W (W = sum |J| + sum |h|, every energy lies in [-W, W]) to the
// entropy density s = ln g(E) / N.  A ladder is placed by the reference's
// constant-acceptance walk (src/cae_estimator.cc:367-425) on the predicted
// ln g instead of a multihistogram estimate from a pilot run.  A short
// pilot then measures the exchange acceptance of the placed ladder; when it
// deviates from the target by more than the tolerance (mean over pairs),
// the ladder is placed again from the measured acceptances (feedback_ladder)
// and measured again, at most three times (none when the first check is off
// by more than 0.2); if it still deviates, the multihistogram ladder
// (pticm_cae_ladder) is used instead.
#include <cuda_runtime.h>

#include <algorithm>
#include <cmath>
#include <cstdio>
#include <cstring>
#include <memory>
#include <string>
#include <vector>

#include "mhist_host.h"
#include "pticm.h"
#include "problem_host.h"
#include "runtime_internal.h"

using namespace pticm;

namespace {

int sfail(int code, const std::string& m) {
    set_last_error(m);
    return code;
}

constexpr int kFeatures = 6;
constexpr double kTargetScale = 10.0;
constexpr int kChecks = 4;   // acceptance checks of a learned ladder: the surrogate's, then up to three feedback placements
constexpr double kHopeless = 0.2;   // a first check this far off goes straight to the multihistogram ladder
constexpr double kOverlapFloor = 0.05;   // lowest pair acceptance for which a check's histograms feed the fallback
constexpr char kMagic[8] = {'P', 'T', 'I', 'C', 'M', 'M', 'L', 'P'};

// ln N / 10, ln M / 12, mean degree / 20, degree std / 10, coupling mean and
// std over the edges (integer couplings as stored).
void features(const HostProblem& P, float* f) {
    const double n = (double)std::max<int64_t>(P.n, 1);
    double m = 0, d1 = 0, d2 = 0, w1 = 0, w2 = 0, cnt = 0;
    for (int64_t i = 0; i < P.n; i++) {
        const double d = (double)(P.row[i + 1] - P.row[i]);
        d1 += d;
        d2 += d * d;
        for (int64_t a = P.row[i]; a < P.row[i + 1]; a++) {
            const double w = (double)P.w[a];
            w1 += w;
            w2 += w * w;
            cnt += 1;
        }
    }
    m = cnt / 2;
    const double dm = d1 / n, dv = std::max(0.0, d2 / n - dm * dm);
    const double wm = cnt > 0 ? w1 / cnt : 0.0, wv = cnt > 0 ? std::max(0.0, w2 / cnt - wm * wm) : 0.0;
    f[0] = (float)(std::log(n) / 10.0);
    f[1] = (float)(std::log(std::max(m, 1.0)) / 12.0);
    f[2] = (float)(dm / 20.0);
    f[3] = (float)(std::sqrt(dv) / 10.0);
    f[4] = (float)wm;
    f[5] = (float)std::sqrt(wv);
}

long long gcdll(long long a, long long b) {
    a = std::llabs(a);
    b = std::llabs(b);
    while (b) { const long long t = a % b; a = b; b = t; }
    return a;
}

// Energy levels of a problem with integer couplings: a flip of site i
// changes E by 2 s_i v_i, v_i = h_i + sum_j J_ij s_j, and every v_i is
// congruent to h_i + sum_j J_ij modulo gcd_j(2 J_ij); so every energy is
// E_up + 2G k with G = gcd_i gcd(h_i + sum_j J_ij, 2 J_ij) and E_up the
// energy of the all-up state.  Returns the step 2G and the lowest level
// >= -W of that class.
void level_grid(const HostProblem& P, long long W, long long& step, long long& first) {
    long long G = 0, eup = 0;
    for (int64_t i = 0; i < P.n; i++) {
        long long v = P.h[i], sumJ = 0;
        for (int64_t a = P.row[i]; a < P.row[i + 1]; a++) {
            sumJ += P.w[a];
            G = gcdll(G, 2 * (long long)P.w[a]);
        }
        v += sumJ;
        G = gcdll(G, v);
        eup += (long long)P.h[i] * 2 + sumJ;   // twice E_up: h counted twice, each edge twice
    }
    eup /= 2;
    if (G == 0) G = 1;
    step = 2 * G;
    long long k = (eup + W) / step;
    first = eup - step * k;
}

// Gaussian (high-temperature) entropy density: ln 2 - E^2 / (2 N V), V the
// energy variance at infinite temperature, sum_e J_e^2 + sum_i h_i^2.  The
// network predicts 10 x (s - this).
double energy_variance(const HostProblem& P) {
    double v = 0;
    for (int64_t i = 0; i < P.n; i++) {
        v += (double)P.h[i] * P.h[i];
        for (int64_t a = P.row[i]; a < P.row[i + 1]; a++) v += 0.5 * (double)P.w[a] * P.w[a];
    }
    return v;
}

// Predicted ln g on the exact levels E = first + step k <= 0.
int predict_levels(const HostProblem& P, pticm_mlp* m, std::vector<double>& lng, long long& W, long long& step,
                   long long& first) {
    W = energy_bound(P);
    if (W <= 0) return sfail(PTICM_ERR_INVALID, "the problem has no couplings");
    level_grid(P, W, step, first);
    if (first > 0) return sfail(PTICM_ERR_INVALID, "no energy level at or below zero");
    const long long nb = (-first) / step + 1;
    float f[kFeatures];
    features(P, f);
    std::vector<float> X((size_t)nb * (kFeatures + 1)), y((size_t)nb);
    for (long long k = 0; k < nb; k++) {
        float* row = X.data() + (size_t)k * (kFeatures + 1);
        std::memcpy(row, f, sizeof f);
        row[kFeatures] = (float)((double)(first + step * k) / (double)W);
    }
    if (int rc = pticm_mlp_predict(m, X.data(), (uint64_t)nb, y.data())) return rc;
    const double n = (double)P.n, V = std::max(energy_variance(P), 1e-12);
    lng.resize((size_t)nb);
    for (long long k = 0; k < nb; k++) {
        const double E = (double)(first + step * k);
        lng[k] = n * std::log(2.0) - E * E / (2.0 * V) + n * (double)y[k] / kTargetScale;
    }
    return PTICM_OK;
}

// The levels where the ladder's temperatures put weight: below the energy
// whose microcanonical beta dS/dE exceeds 2 beta_max, or above the one where
// it falls under beta_min / 2, exp(S - beta E) decays at least as
// exp(-beta_max |dE|) away from the kept range for every beta of the ladder.
void cut_range(const std::vector<double>& lng, double estep, double beta_max, double beta_min, size_t& lo,
               size_t& hi) {
    const size_t nb = lng.size();
    lo = 0;
    hi = nb - 1;
    if (nb < 3) return;
    auto slope = [&](size_t k) { return (lng[k + 1] - lng[k - 1]) / (2 * estep); };
    size_t k = nb - 2;
    while (k > 1 && slope(k) <= 2 * beta_max) k--;
    lo = k;
    k = lo + 1;
    while (k < nb - 2 && slope(k) >= 0.5 * beta_min) k++;
    hi = std::max(k, lo + 2);
    hi = std::min(hi, nb - 1);
}

// erfc^-1(a), a in (0, 2): Newton steps on std::erfc from a bracketed start.
double erfc_inv(double a) {
    a = std::min(std::max(a, 1e-300), 2.0 - 1e-16);
    double y = a < 1 ? std::sqrt(-std::log(a / 2)) * 0.7 : -std::sqrt(-std::log((2 - a) / 2)) * 0.7;
    for (int it = 0; it < 60; it++) {
        const double f = std::erfc(y) - a;
        const double d = -1.1283791670955126 * std::exp(-y * y);   // d erfc / dy = -2/sqrt(pi) e^{-y^2}
        if (d == 0) break;
        const double step = f / d;
        y -= step;
        if (std::fabs(step) < 1e-12 * (1 + std::fabs(y))) break;
    }
    return y;
}

// Feedback placement: a measured acceptance A_k of the gap between b_k and
// b_{k+1} gives the energy spread there, sigma_k = 2 erfc^-1(A_k) / dbeta
// (exchange between Gaussian energy distributions of equal width sigma is
// accepted with probability erfc(dbeta sigma / 2)); the new ladder walks from
// the coldest temperature with dbeta = 2 erfc^-1(r) / sigma(beta) until it
// passes beta_end (then beta_end) or holds nt temperatures.  A gap without
// accepted exchanges counts as A = 1 / (2 (attempts + 1)).
std::vector<double> feedback_ladder(const std::vector<double>& lad, const std::vector<double>& acc, double attempts,
                                    double r, uint32_t nt, double beta_end) {
    const size_t g = acc.size();
    std::vector<double> sig(g);
    for (size_t k = 0; k < g; k++) {
        const double a = std::min(std::max(acc[k], 0.5 / (attempts + 1)), 1.0 - 0.5 / (attempts + 1));
        sig[k] = 2 * erfc_inv(a) / std::max(lad[k] - lad[k + 1], 1e-12);
    }
    const double target = 2 * erfc_inv(r);
    std::vector<double> out{lad[0]};
    double b = lad[0];
    size_t k = 0;
    while (out.size() < nt) {
        while (k + 1 < g && b <= lad[k + 1]) k++;
        const double nb = b - target / sig[k];
        if (nb <= beta_end) {
            out.push_back(beta_end);
            break;
        }
        out.push_back(nb);
        b = nb;
    }
    return out;
}

}  // namespace

extern "C" {

int pticm_problem_features(const pticm_problem* p, float* out) {
    if (!p || !out) return sfail(PTICM_ERR_INVALID, "null argument");
    features(problem_host(p), out);
    return PTICM_OK;
}

int pticm_surrogate_logdos(const pticm_problem* p, pticm_mlp* m, double* logdos, uint64_t cap, uint64_t* nbins,
                           double* emin, double* estep) {
    if (!p || !m || !nbins) return sfail(PTICM_ERR_INVALID, "null argument");
    std::vector<double> lng;
    long long W = 0, step = 0, first = 0;
    if (int rc = predict_levels(problem_host(p), m, lng, W, step, first)) return rc;
    *nbins = lng.size();
    if (emin) *emin = (double)first;
    if (estep) *estep = (double)step;
    if (logdos) {
        if (cap < lng.size()) return sfail(PTICM_ERR_INVALID, "logdos buffer too small");
        std::copy(lng.begin(), lng.end(), logdos);
    }
    return PTICM_OK;
}

int pticm_surrogate_ladder(const pticm_problem* p, pticm_mlp* m, double T0, double T1, int inverse, uint32_t nt,
                           double step_size, double r, double* beta_out, uint32_t* count) {
    if (!p || !m || !beta_out || !count || nt < 2) return sfail(PTICM_ERR_INVALID, "invalid arguments");
    double bs = inverse ? T0 : 1 / T0, be = inverse ? T1 : 1 / T1;
    if (bs < be) std::swap(bs, be);
    std::vector<double> lng;
    long long W = 0, step = 0, first = 0;
    if (int rc = predict_levels(problem_host(p), m, lng, W, step, first)) return rc;
    size_t lo = 0, hi = 0;
    cut_range(lng, (double)step, bs, be, lo, hi);
    // no level holds fewer than one state: ln g >= 0 bounds the spectrum
    while (lo + 2 < hi && lng[lo] < 0) lo++;
    std::vector<double> dos(lng.begin() + lo, lng.begin() + hi + 1);
    *count = cae_walk(dos, (double)(first + step * (long long)lo), (double)step, bs, be, step_size, r, nt, beta_out);
    return PTICM_OK;
}

}  // extern "C"

namespace {

// A PT run (two chains, no ICM) on a ladder: the exchange acceptance of each
// neighbouring pair over `steps` steps after `burn_in`, and, when `hist` is
// given, the per-slot energy histograms of those steps (R rows of nbins
// bins, bin b at energy lo + 2b).
int ladder_check(const pticm_problem* p, const double* beta, uint32_t nt, uint64_t seed, uint64_t steps,
                 uint64_t burn_in, double* acc, std::vector<unsigned>* hist, int64_t* lo, uint64_t* nbins) {
    pticm_opts o;
    pticm_opts_default(&o);
    o.seed = seed;
    o.nt = nt;
    o.chains = 2;
    o.icm = 0;
    pticm_ctx* c = nullptr;
    if (int rc = pticm_create(p, &o, &c)) return rc;
    std::unique_ptr<pticm_ctx, void (*)(pticm_ctx*)> hold(c, pticm_destroy);
    if (int rc = pticm_set_ladder(c, beta, nt, 0)) return rc;
    if (int rc = pticm_init_states(c, seed)) return rc;
    if (hist)
        if (int rc = pticm_enable_energy_histograms(c, burn_in)) return rc;
    std::vector<uint64_t> a0(2 * nt), s0(2 * nt), a1(2 * nt), s1(2 * nt);
    if (burn_in)
        if (int rc = pticm_run(c, burn_in, PTICM_PHASE_SWEEP | PTICM_PHASE_EXCHANGE)) return rc;
    if (int rc = pticm_get_stats(c, nullptr, a0.data(), s0.data())) return rc;
    if (int rc = pticm_run(c, steps, PTICM_PHASE_SWEEP | PTICM_PHASE_EXCHANGE)) return rc;
    if (int rc = pticm_get_stats(c, nullptr, a1.data(), s1.data())) return rc;
    for (uint32_t k = 0; k + 1 < nt; k++) {
        const double at = (double)(a1[k] - a0[k] + a1[k + nt] - a0[k + nt]);
        const double su = (double)(s1[k] - s0[k] + s1[k + nt] - s0[k + nt]);
        acc[k] = at > 0 ? su / at : 0.0;
    }
    if (hist) {
        if (int rc = pticm_get_energy_histograms(c, nullptr, lo, nbins)) return rc;
        hist->assign((size_t)(2 * nt) * (size_t)*nbins, 0u);
        if (int rc = pticm_get_energy_histograms(c, hist->data(), lo, nbins)) return rc;
    }
    return PTICM_OK;
}

}  // namespace

extern "C" {

int pticm_ladder_acceptance(const pticm_problem* p, const double* beta, uint32_t nt, uint64_t seed, uint64_t steps,
                            uint64_t burn_in, double* acc) {
    if (!p || !beta || !acc || nt < 2 || steps == 0) return sfail(PTICM_ERR_INVALID, "invalid arguments");
    return ladder_check(p, beta, nt, seed, steps, burn_in, acc, nullptr, nullptr, nullptr);
}

int pticm_learned_ladder(const pticm_problem* p, pticm_mlp* m, double T0, double T1, int inverse, uint32_t nt,
                         double r, uint64_t check_steps, double tol, uint64_t seed, double* beta_out,
                         uint32_t* count, pticm_learned_ladder_info* info) {
    if (!p || !m || !beta_out || !count || nt < 2) return sfail(PTICM_ERR_INVALID, "invalid arguments");
    pticm_learned_ladder_info li{};
    std::vector<double> lad(nt);
    uint32_t cnt = 0;
    if (int rc = pticm_surrogate_ladder(p, m, T0, T1, inverse, nt, 0.1, r, lad.data(), &cnt)) return rc;
    lad.resize(cnt);
    li.surrogate_count = cnt;
    bool ok = cnt >= 2;
    double be = inverse ? T1 : 1 / T1, bs = inverse ? T0 : 1 / T0;
    if (bs < be) std::swap(bs, be);
    // the energy histograms of the last check, and its ladder: the
    // multihistogram fallback's samples
    std::vector<unsigned> hist;
    std::vector<double> hist_beta;
    int64_t hist_lo = 0;
    uint64_t hist_nbins = 0;
    double hist_min_acc = 0.0;   // the lowest pair acceptance of that check
    for (int round = 0; ok && check_steps > 0 && round < kChecks; round++) {
        std::vector<double> acc(lad.size() - 1);
        if (int rc = ladder_check(p, lad.data(), (uint32_t)lad.size(), seed + round, check_steps, check_steps / 4,
                                  acc.data(), &hist, &hist_lo, &hist_nbins))
            return rc;
        hist_beta = lad;
        hist_min_acc = acc.empty() ? 0.0 : *std::min_element(acc.begin(), acc.end());
        double dev = 0;
        for (double a : acc) dev += std::fabs(a - r);
        li.mean_deviation = dev / (double)acc.size();
        li.rounds = round + 1;
        if (round == 0) li.first_deviation = li.mean_deviation;
        if (li.mean_deviation <= tol || round == kChecks - 1) break;
        if (round == 0 && li.mean_deviation > kHopeless) break;
        // feedback re-placement from the measured acceptances
        std::vector<double> out = feedback_ladder(lad, acc, (double)check_steps, r, nt, be);
        li.inserted += (uint32_t)(out.size() > lad.size() ? out.size() - lad.size() : 0);
        lad = out;
        ok = lad.size() >= 2;
    }
    ok = ok && li.mean_deviation <= tol;
    if (ok) {
        std::copy(lad.begin(), lad.end(), beta_out);
        *count = (uint32_t)lad.size();
    } else {
        li.fallback = 1;
        // the multihistogram ladder (src/cae_estimator.cc:155-428) from the
        // samples the checks already drew: the last check's two chains at
        // its temperatures, when every neighbouring pair of them exchanged
        // often enough for their histograms to overlap; otherwise a
        // separate pilot run (pticm_cae_ladder)
        std::vector<double> dos, z;
        double min_emin = 0;
        uint64_t it = 0;
        if (!hist.empty() && hist_min_acc >= kOverlapFloor &&
            slot_hist_dos(hist.data(), (int)hist_beta.size(), 2, (long long)hist_nbins, (long long)hist_lo,
                          hist_beta.data(), 2.0, dos, z, min_emin, it) == PTICM_OK) {
            *count = cae_walk(dos, min_emin, 2.0, bs, be, 0.1, r, nt, beta_out);
        } else if (int rc = pticm_cae_ladder(p, seed, T0, T1, inverse, nt, 2.0, 0.1, r, 2000, 5000, beta_out,
                                             count)) {
            return rc;
        }
    }
    if (info) *info = li;
    return PTICM_OK;
}

int pticm_feedback_ladder(const double* beta, uint32_t count, const double* acc, double attempts, double r,
                          uint32_t nt, double beta_end, double* beta_out, uint32_t* out_count) {
    if (!beta || !acc || !beta_out || !out_count || count < 2 || nt < 2)
        return sfail(PTICM_ERR_INVALID, "invalid arguments");
    std::vector<double> lad(beta, beta + count), a(acc, acc + count - 1);
    std::vector<double> out = feedback_ladder(lad, a, attempts, r, nt, beta_end);
    std::copy(out.begin(), out.end(), beta_out);
    *out_count = (uint32_t)out.size();
    return PTICM_OK;
}

int pticm_mlp_save(pticm_mlp* m, const char* path) {
    if (!m || !path) return sfail(PTICM_ERR_INVALID, "null argument");
    const uint64_t n = pticm_mlp_param_count();
    std::vector<float> p(n);
    if (int rc = pticm_mlp_get_params(m, p.data())) return rc;
    FILE* f = std::fopen(path, "wb");
    if (!f) return sfail(PTICM_ERR_IO, std::string("cannot write ") + path);
    const uint32_t version = 1;
    bool ok = std::fwrite(kMagic, 1, 8, f) == 8 && std::fwrite(&version, 4, 1, f) == 1 &&
              std::fwrite(&n, 8, 1, f) == 1 && std::fwrite(p.data(), 4, n, f) == n;
    ok = (std::fclose(f) == 0) && ok;
    return ok ? PTICM_OK : sfail(PTICM_ERR_IO, std::string("short write to ") + path);
}

int pticm_mlp_load(pticm_mlp* m, const char* path) {
    if (!m || !path) return sfail(PTICM_ERR_INVALID, "null argument");
    FILE* f = std::fopen(path, "rb");
    if (!f) return sfail(PTICM_ERR_IO, std::string("cannot read ") + path);
    char magic[8];
    uint32_t version = 0;
    uint64_t n = 0;
    const uint64_t want = pticm_mlp_param_count();
    std::vector<float> p(want);
    bool ok = std::fread(magic, 1, 8, f) == 8 && std::memcmp(magic, kMagic, 8) == 0 && std::fread(&version, 4, 1, f) == 1 &&
              version == 1 && std::fread(&n, 8, 1, f) == 1 && n == want && std::fread(p.data(), 4, n, f) == n;
    std::fclose(f);
    if (!ok) return sfail(PTICM_ERR_IO, std::string(path) + " is not a surrogate network file of this version");
    return pticm_mlp_set_params(m, p.data());
}

}  // extern "C"
