// shim_driver.cc -- code written in the reference's shape, compiled against
// the libreplica interface of this library (pt-icm_gb300/host/pticm_gb300.hh)
// by tests/test_gpu_shim.py.
//
//   shim_driver solve GRAPH SEED NT PTS ICM T0 T1 SWEEPS
//       read_problem, initialize_*, then the main loop of the reference's
//       solve() (src/solver.cc:67-127) over Replica::sweep,
//       try_replica_exchange and icm; prints the report keys, the final
//       replica states and energies
//   shim_driver pilot GRAPH SEED NT SAMPLES BURN_IN T0 T1
//       the pilot loop of get_beta's gather_samples
//       (src/cae_estimator.cc:76-140): one chain of Replica objects on the
//       linear-beta ladder, shuffled exchanges; prints per temperature the
//       sample count, the sums of E and E^2, and the extreme energies
#include <algorithm>
#include <cmath>
#include <cstdio>
#include <cstdlib>
#include <string>
#include <vector>

#include "pticm_gb300.hh"

using namespace pticm;

static void print_u32(const char* key, const std::vector<uint32_t>& v) {
    std::printf("%s:", key);
    for (uint32_t x : v) std::printf(" %u", x);
    std::printf("\n");
}

static int run_solve(int argc, char** argv) {
    if (argc < 10) return 2;
    PTWorker w;
    w.params.seed = std::strtoull(argv[3], nullptr, 10);
    w.params.Nt = std::strtoull(argv[4], nullptr, 10);
    w.params.pts = std::strtoull(argv[5], nullptr, 10);
    w.params.icm = std::atoi(argv[6]) != 0;
    w.params.T0 = std::atof(argv[7]);
    w.params.T1 = std::atof(argv[8]);
    w.params.sweeps = std::strtoull(argv[9], nullptr, 10);
    std::string path = argv[2];
    read_problem(w, path);
    initialize_temperatures(w);
    initialize_replicas(w);
    initialize_replica_exchanges(w);
    // MAIN MCMC LOOP (the shape of src/solver.cc:67-127)
    for (size_t i = 0; i < w.params.pts; i++) {
        for (size_t s = 0; s < w.params.sweeps; s++) {
            uint64_t replica_ind = 0;
            for (Replica& r : w.replicas) {
                r.sweep(w.p);
                w.energy_values_local[replica_ind++] = r.get_energy();
            }
        }
        gather_energy_values(w);
        for (size_t m = 0; m < w.params.Nt - 1; m++) {
            if (w.wid == 0) {
                try_replica_exchange(w, 0);
                try_replica_exchange(w, 1);
            } else {
                check_for_replica_exchange(w);
                check_for_replica_exchange(w);
            }
        }
        if (w.params.icm) {
            for (int icm_target = (int)w.params.Nt - 1; icm_target >= static_cast<int>(w.params.Nt - w.Nc);
                 icm_target--) {
                if (w.wid == 0) icm(w, icm_target);
                else check_icm(w);
            }
        }
    }
    double best_ene = 0.0;
    size_t best_sweep = 0;
    StateVector best_state;
    gather_best_energy_values(w, best_ene, best_sweep, best_state);
    const uint64_t flips = get_flips(w);
    print_u32("swap_attempts", w.swap_attempts);
    print_u32("swap_successes", w.swap_successes);
    std::printf("best_energy: %.17g\n", best_ene);
    std::printf("best_sweep: %zu\n", best_sweep);
    std::printf("best_maxcut: %.17g\n", w.p.maxcut(best_state));
    std::printf("num_of_flips: %llu\n", (unsigned long long)flips);
    std::printf("num_of_swaps: %llu\n", (unsigned long long)w.swaps);
    std::printf("nc: %u\n", w.Nc);
    std::printf("best_state: ");
    for (bool b : best_state) std::printf("%d", b ? 1 : 0);
    std::printf("\n");
    for (size_t r = 0; r < w.replicas.size(); r++) {
        std::printf("replica %zu %.17g ", r, w.replicas[r].get_energy());
        for (bool b : w.replicas[r].get_state()) std::printf("%d", b ? 1 : 0);
        std::printf("\n");
    }
    // the incremental dE update of one flip against a from-scratch one
    const StateVector& s0 = w.replicas[0].get_state();
    std::vector<double> dE = w.replicas[0].get_dE(), fresh;
    w.p.incremental_dE(dE, s0, 0);
    StateVector s1 = s0;
    s1[0] = !s1[0];
    w.p.calculate_dE(fresh, s1);
    std::printf("incremental_dE_matches: %d\n", dE == fresh ? 1 : 0);
    return 0;
}

static int run_pilot(int argc, char** argv) {
    if (argc < 9) return 2;
    PTWorker w;
    w.params.seed = std::strtoull(argv[3], nullptr, 10);
    const size_t Nt = std::strtoull(argv[4], nullptr, 10);
    const size_t num_samples = std::strtoull(argv[5], nullptr, 10);
    const size_t BURN_IN = std::strtoull(argv[6], nullptr, 10);
    const double T0 = std::atof(argv[7]), T1 = std::atof(argv[8]);
    read_problem(w, argv[2]);
    // the pilot ladder of get_beta (src/cae_estimator.cc:308-328)
    double beta_start = 1 / T0, beta_end = 1 / T1;
    if (beta_start < beta_end) std::swap(beta_start, beta_end);
    std::vector<double> beta_values(Nt);
    const double beta_step = (beta_end - beta_start) / (double)(Nt - 1);
    double beta = beta_start;
    for (size_t i = 0; i < Nt; i++, beta += beta_step) beta_values[i] = beta;
    // gather_samples (the shape of src/cae_estimator.cc:76-140)
    uint64_t N = w.p.vcount();
    StateVector init_state(N);
    std::bernoulli_distribution bern(0.5);
    std::vector<Replica> chain(Nt);
    std::vector<unsigned> swap_order(Nt - 1);
    std::vector<unsigned> replica_inds(Nt);
    std::vector<std::vector<double>> energylogs(Nt);
    size_t ind = 0;
    for (auto& r : chain) {
        energylogs[ind].reserve(num_samples);
        replica_inds[ind] = (unsigned)ind;
        if (ind < Nt - 1) swap_order[ind] = (unsigned)ind;
        for (size_t i = 0; i < N; i++) init_state[i] = bern(w.p.get_rng());
        std::vector<double> dE(N, 0);
        double ene_start = w.p.calculate_dE(dE, init_state);
        r = Replica(w.p, beta_values[ind++], init_state, dE, ene_start, false, BURN_IN);
    }
    for (size_t i = 0; i < BURN_IN + num_samples; i++) {
        for (size_t rind = 0; rind < Nt; rind++) {
            Replica& r = chain[replica_inds[rind]];
            r.sweep(w.p);
            if (i >= BURN_IN) energylogs[rind].push_back(r.get_energy());
        }
        std::shuffle(swap_order.begin(), swap_order.end(), w.p.get_rng());
        for (auto index : swap_order) {
            Replica& r1 = chain[replica_inds[index]];
            Replica& r2 = chain[replica_inds[index + 1]];
            double e1 = r1.get_energy();
            double e2 = r2.get_energy();
            double beta1 = beta_values[index];
            double beta2 = beta_values[index + 1];
            double logboltz = (e1 - e2) * (beta1 - beta2);
            double rngnum = w.p.rand_double();
            if (std::log(rngnum) < logboltz) {
                std::swap(replica_inds[index], replica_inds[index + 1]);
                r1.set_beta(beta2);
                r2.set_beta(beta1);
            }
        }
    }
    for (size_t j = 0; j < Nt; j++) {
        const std::vector<double>& L = energylogs[j];
        double s = 0, s2 = 0;
        for (double e : L) { s += e; s2 += e * e; }
        std::printf("pilot %zu %zu %.17g %.17g %.17g %.17g\n", j, L.size(), s, s2,
                    *std::min_element(L.begin(), L.end()), *std::max_element(L.begin(), L.end()));
    }
    return 0;
}

int main(int argc, char** argv) {
    if (argc < 2) return 2;
    try {
        if (std::string(argv[1]) == "solve") return run_solve(argc, argv);
        if (std::string(argv[1]) == "pilot") return run_pilot(argc, argv);
    } catch (const std::exception& e) {
        std::fprintf(stderr, "%s\n", e.what());
        return 1;
    }
    return 2;
}
