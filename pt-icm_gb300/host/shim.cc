// shim.cc -- the reference's C++ interface over the GB300 engine's C ABI.
#include <algorithm>
#include <memory>
#include <charconv>
#include <chrono>
#include <cstdio>
#include <stdexcept>
#include <string>

#include "pticm_gb300.hh"

namespace pticm {

namespace {

void check(int rc) {
    if (rc != PTICM_OK) throw std::runtime_error(std::string("pticm: ") + pticm_last_error());
}

std::vector<uint8_t> to_bytes(const StateVector& s) { return std::vector<uint8_t>(s.begin(), s.end()); }

// fmt's "{}" for a double: the shortest representation that round-trips
std::string shortest(double v) {
    char buf[64];
    auto r = std::to_chars(buf, buf + sizeof(buf), v);
    return std::string(buf, r.ptr);
}

}  // namespace

// ------------------------------------------------------------------ Problem
Problem::Problem(std::string path, uint64_t seed, uint64_t burn_in) : seed_(seed), burn_in_(burn_in), rng_(seed) {
    check(pticm_problem_load_gset(path.c_str(), &h_));
    refresh();
}

Problem::Problem(double* weights, int* src, int* dest, double* linear, uint64_t seed, uint64_t burn_in, uint64_t N,
                 uint64_t M)
    : seed_(seed), burn_in_(burn_in), rng_(seed) {
    std::vector<int32_t> s(src, src + M), d(dest, dest + M);
    check(pticm_problem_from_coo((int64_t)N, (int64_t)M, s.data(), d.data(), weights, linear, &h_));
    refresh();
}

Problem::Problem(double* formulation, double* linear, uint64_t seed, uint64_t burn_in, uint64_t N)
    : seed_(seed), burn_in_(burn_in), rng_(seed) {
    check(pticm_problem_from_dense((int64_t)N, formulation, linear, &h_));
    refresh();
}

Problem::Problem(Problem&& o) noexcept
    : h_(o.h_), info_(o.info_), seed_(o.seed_), burn_in_(o.burn_in_), rng_(o.rng_), unif_(o.unif_) {
    o.h_ = nullptr;
}

Problem& Problem::operator=(Problem&& o) noexcept {
    if (this != &o) {
        if (h_) pticm_problem_free(h_);
        h_ = o.h_;
        info_ = o.info_;
        seed_ = o.seed_;
        burn_in_ = o.burn_in_;
        rng_ = o.rng_;
        unif_ = o.unif_;
        o.h_ = nullptr;
    }
    return *this;
}

Problem::~Problem() {
    if (h_) pticm_problem_free(h_);
}

void Problem::refresh() { check(pticm_problem_get_info(h_, &info_)); }

double Problem::energy(const StateVector& s) const {
    auto b = to_bytes(s);
    double E = 0, cut = 0;
    check(pticm_problem_evaluate(h_, 1, b.data(), &E, &cut, nullptr));
    return E;
}

double Problem::energy(bool* s) const { return energy(StateVector(s, s + vcount())); }

void Problem::incremental_dE(std::vector<double>& dE, const StateVector& s, uint32_t index) const {
    auto b = to_bytes(s);
    dE.resize(s.size());
    check(pticm_problem_incremental_dE(h_, dE.data(), b.data(), index));
}

double Problem::maxcut(const StateVector& s) const {
    auto b = to_bytes(s);
    double E = 0, cut = 0;
    check(pticm_problem_evaluate(h_, 1, b.data(), &E, &cut, nullptr));
    return cut;
}

double Problem::calculate_dE(std::vector<double>& dE, const StateVector& s) const {
    auto b = to_bytes(s);
    dE.resize(s.size());
    double E = 0, cut = 0;
    check(pticm_problem_evaluate(h_, 1, b.data(), &E, &cut, dE.data()));
    return E;
}

// ------------------------------------------------------------------ worker
PTWorker::~PTWorker() {
    if (ctx) pticm_destroy(ctx);
}

void beta_linspace(double* temps, double T0, double T1, uint64_t num_temp, bool inverse) {
    check(pticm_beta_linspace(temps, T0, T1, num_temp, inverse ? 1 : 0));
}

void get_beta(PTWorker& w, double estep, double step_size, double r, size_t num_samples) {
    std::vector<double> beta(w.params.Nt);
    uint32_t count = 0;
    check(pticm_cae_ladder(w.p.handle(), w.params.seed, w.params.T0, w.params.T1, w.params.inverse ? 1 : 0,
                           (uint32_t)w.params.Nt, estep, step_size, r, num_samples, 5000, beta.data(), &count));
    beta.resize(count);
    w.params.Nt = count;
    w.beta_values = beta;
}

// The learned ladder: the surrogate network's constant-acceptance ladder,
// checked by a short PT run, with the multihistogram ladder as fallback.
void learned_beta(PTWorker& w, double r) {
    pticm_mlp* m = nullptr;
    check(pticm_mlp_create(w.params.seed, 1024, &m));
    std::unique_ptr<pticm_mlp, void (*)(pticm_mlp*)> hold(m, pticm_mlp_destroy);
    check(pticm_mlp_load(m, w.params.learned_ladder.c_str()));
    std::vector<double> beta(w.params.Nt);
    uint32_t count = 0;
    pticm_learned_ladder_info info{};
    check(pticm_learned_ladder(w.p.handle(), m, w.params.T0, w.params.T1, w.params.inverse ? 1 : 0,
                               (uint32_t)w.params.Nt, r, 1000, 0.05, w.params.seed, beta.data(), &count, &info));
    beta.resize(count);
    w.params.Nt = count;
    w.beta_values = beta;
    if (w.params.verbosity)
        std::printf("learned ladder: %u temperatures, %s (mean |acceptance - r| %.3f after %u checks)\n", count,
                    info.fallback ? "multihistogram fallback" : "accepted", info.mean_deviation, info.rounds);
}

void choose_ladder(PTWorker& w) {
    w.characteristic_scale = w.p.get_char_scale();
    if (!w.params.learned_ladder.empty()) {
        learned_beta(w, 0.4);
        if (w.params.sort_ladder) std::sort(w.beta_values.begin(), w.beta_values.end());
    } else if (w.params.preprocess) {
        get_beta(w, 2, w.params.pre_step, 0.4, w.params.pre_samples);
        if (w.params.sort_ladder) std::sort(w.beta_values.begin(), w.beta_values.end());
    } else {
        w.beta_values.assign(w.params.Nt, 0.0);
        beta_linspace(w.beta_values.data(), w.params.T0, w.params.T1, w.params.Nt, w.params.inverse);
    }
}

void initialize_temperatures(PTWorker& w) {
    choose_ladder(w);
    pticm_opts o;
    pticm_opts_default(&o);
    o.seed = w.params.seed;
    o.nt = (uint32_t)w.params.Nt;
    o.chains = w.params.chains;
    o.sweeps = (uint32_t)w.params.sweeps;
    o.icm = w.params.icm ? 1 : 0;
    o.exchange = w.params.exchange;
    o.best_per_phase = w.params.best_per_phase;
    o.replicas_per_block = w.params.replicas_per_block;
    o.block_threads = w.params.block_threads;
    o.icm_algo = w.params.icm_algo;
    if (w.ctx) pticm_destroy(w.ctx);
    w.ctx = nullptr;
    check(pticm_create(w.p.handle(), &o, &w.ctx));
    check(pticm_set_ladder(w.ctx, w.beta_values.data(), (uint32_t)w.params.Nt, -1));
    // src/initialization.cc:158-164: the pairs counted from the top slot down
    // while beta >= the characteristic scale, whether or not ICM is on
    w.Nc = 0;
    for (int64_t i = (int64_t)w.params.Nt - 1; i >= 0; i--) {
        if (w.beta_values[(size_t)i] < w.characteristic_scale) break;
        w.Nc++;
    }
    const size_t R = (size_t)w.params.Nt * w.params.chains;
    std::vector<double> doubled;
    for (uint32_t c = 0; c < w.params.chains; c++) doubled.insert(doubled.end(), w.beta_values.begin(), w.beta_values.end());
    w.beta_values = doubled;
    w.beta_indices.assign(R, 0);
    for (size_t k = 0; k < R; k++) w.beta_indices[k] = (uint32_t)k;
    w.swap_attempts.assign(R, 0);
    w.swap_successes.assign(R, 0);
    // one worker holds every replica: replica i is in chain i / Nt at slot i
    // (src/initialization.cc:120-172 with numw = 1)
    w.worker_r = w.last_r = w.loc_r = R;
    w.replica_workers.assign(R, 0);
    w.chain_index_global.assign(R, 0);
    for (size_t i = 0; i < R; i++) w.chain_index_global[i] = (uint8_t)(i / w.params.Nt);
    w.chain_index_local = w.chain_index_global;
    w.beta_values_local = w.beta_values;
}

void sweep_all(PTWorker& w) { check(pticm_run(w.ctx, 1, PTICM_PHASE_SWEEP)); }
void replica_exchange(PTWorker& w) { check(pticm_run(w.ctx, 1, PTICM_PHASE_EXCHANGE)); }
void icm_all(PTWorker& w) { check(pticm_run(w.ctx, 1, PTICM_PHASE_ICM)); }

void gather_best_energy_values(PTWorker& w, double& best_ene, size_t& best_sweep, StateVector& best_state) {
    if (!w.replicas.empty()) {
        // src/mpi_utils.cc:103-163 over the worker's Replica objects: the
        // first replica with the lowest best energy
        best_ene = 1.7976931348623157e308;
        best_sweep = 0;
        for (Replica& r : w.replicas) {
            const double e = r.get_best_ene();
            if (e < best_ene) {
                best_ene = e;
                best_state = r.get_best_state();
                best_sweep = r.get_best_sweep();
            }
        }
        return;
    }
    std::vector<uint8_t> s(w.p.vcount());
    uint64_t sweep = 0;
    int64_t rep = -1;
    check(pticm_get_best(w.ctx, &best_ene, &sweep, s.data(), &rep));
    best_sweep = (size_t)sweep;
    best_state.assign(s.begin(), s.end());
}

uint64_t get_flips(PTWorker& w) {
    if (!w.replicas.empty()) {
        // src/mpi_utils.cc:167-176 (summed in 64 bits: the reference's int
        // accumulator wraps past 2^31)
        uint64_t sum = 0;
        for (const Replica& r : w.replicas) sum += r.get_flips();
        return sum;
    }
    pticm_stats st;
    check(pticm_get_stats(w.ctx, &st, nullptr, nullptr));
    return st.flips;
}

static void refresh_exchange(PTWorker& w) {
    const size_t R = w.beta_indices.size();
    std::vector<uint64_t> att(R), suc(R);
    pticm_stats st;
    check(pticm_get_stats(w.ctx, &st, att.data(), suc.data()));
    for (size_t k = 0; k < R; k++) {
        w.swap_attempts[k] = (uint32_t)att[k];
        w.swap_successes[k] = (uint32_t)suc[k];
    }
    w.swaps = st.swaps;
    check(pticm_get_ladder(w.ctx, nullptr, w.beta_indices.data(), nullptr));
}

void solve(PTWorker& w, std::string& problem_path, double& best_ene, size_t& flips, StateVector& best_state) {
    const auto t0 = std::chrono::steady_clock::now();
    read_problem(w, problem_path);
    w.replicas.clear();
    initialize_temperatures(w);
    bool have_hist = false;
    if (!w.params.resume.empty()) {
        // continue a checkpointed run: its ladder, replicas, counters and
        // step count replace the fresh ones (a context of the same problem
        // and options is required)
        check(pticm_checkpoint_load(w.ctx, w.params.resume.c_str()));
        const size_t nt = (size_t)w.params.Nt;
        check(pticm_get_ladder(w.ctx, w.beta_values.data(), nullptr, nullptr));
        for (uint32_t c = 1; c < w.params.chains; c++)
            std::copy(w.beta_values.begin(), w.beta_values.begin() + nt, w.beta_values.begin() + c * nt);
        int64_t lo = 0;
        uint64_t nb = 0;
        have_hist = pticm_get_energy_histograms(w.ctx, nullptr, &lo, &nb) == PTICM_OK;
    } else {
        // the GPU-resident run draws its initial states on the device
        check(pticm_init_states(w.ctx, w.params.seed));
    }
    // --log: per-temperature observables from the steps after the burn-in
    if (w.params.log_data && !have_hist) check(pticm_enable_energy_histograms(w.ctx, w.params.burn_in));
    check(pticm_run(w.ctx, w.params.pts, PTICM_PHASE_ALL));
    if (!w.params.checkpoint.empty()) check(pticm_checkpoint_save(w.ctx, w.params.checkpoint.c_str()));
    size_t best_sweep = 0;
    gather_best_energy_values(w, best_ene, best_sweep, best_state);
    flips = (size_t)get_flips(w);
    refresh_exchange(w);
    const double elapsed = std::chrono::duration<double>(std::chrono::steady_clock::now() - t0).count();
    // the report of src/solver.cc:151-163
    const size_t R = w.swap_attempts.size();
    std::string line = "swap_rates: [";
    for (size_t k = 0; k < R; k++) {
        char b[64];
        const double rate = w.swap_attempts[k] ? (double)w.swap_successes[k] / w.swap_attempts[k] : 0.0;
        std::snprintf(b, sizeof b, "%s%.6f", k ? ", " : "", rate);
        line += b;
    }
    std::printf("%s]\n", line.c_str());
    auto print_u = [&](const char* key, const std::vector<uint32_t>& v) {
        std::string s = std::string(key) + ": [";
        for (size_t k = 0; k < v.size(); k++) s += (k ? ", " : "") + std::to_string(v[k]);
        std::printf("%s]\n", s.c_str());
    };
    print_u("swap_attempts", w.swap_attempts);
    print_u("swap_successes", w.swap_successes);
    std::printf("best_state_energy: %s\n", shortest(w.p.energy(best_state)).c_str());
    std::printf("best_state_sweep: %zu\n", best_sweep);
    std::printf("best_energy: %s \n", shortest(best_ene).c_str());
    std::printf("best_maxcut: %s\n", shortest(w.p.maxcut(best_state)).c_str());
    std::printf("num_of_flips: %zu\n", flips);
    std::printf("num_of_swaps: %llu\n", (unsigned long long)w.swaps);
    std::string bs = "best_state: [", bits;
    for (size_t i = 0; i < best_state.size(); i++) {
        bs += (i ? ", " : "") + std::string(best_state[i] ? "1" : "0");
        bits += best_state[i] ? '1' : '0';
    }
    std::printf("%s]\n%s\n", bs.c_str(), bits.c_str());
    std::string lad = "[";
    for (size_t k = 0; k < (size_t)w.params.Nt; k++) {
        char b[64];
        std::snprintf(b, sizeof b, "%s%.6f", k ? ", " : "", w.beta_values[k]);
        lad += b;
    }
    std::printf("%s]\n", lad.c_str());
    std::printf("Total time: %.6f\n", elapsed);
    std::fflush(stdout);
    if (w.params.log_data) {
        // the table the reference's --log was to write (src/main.cc:490-530): T,C,X,u,m
        const size_t nt = (size_t)w.params.Nt;
        std::vector<double> T(nt), C(nt), X(nt), U(nt), M(nt);
        std::vector<uint64_t> ns(nt);
        check(pticm_get_observables(w.ctx, T.data(), C.data(), X.data(), U.data(), M.data(), ns.data()));
        std::printf("T,C,X,u,m\n");
        for (size_t k = 0; k < nt; k++) std::printf("%f,%f,%f,%f,%f\n", T[k], C[k], X[k], U[k], M[k]);
    }
}

}  // namespace pticm
