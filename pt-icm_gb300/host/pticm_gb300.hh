// pticm_gb300.hh -- the reference's C++ interface (the libreplica headers
// problem.hh, replica.hh, replica_exchange.hh, icm.hh, initialization.hh,
// solver.hh, mpi_utils.hh, utils.hh and mpi_defs.hh) over the GB300 engine's
// C ABI (include/pticm.h).
//
// Two layers share the names:
//  * the per-replica layer: Replica (its sweep runs on the GPU),
//    try_replica_exchange, icm, xor_icm, bfs_icm, Problem::incremental_dE and
//    the initialisation functions keep the reference's signatures, argument
//    meanings, random-number draws and results.  Code written in the
//    reference's shape -- its solve loop (src/solver.cc:67-127), get_beta's
//    pilot loop (src/cae_estimator.cc:112-140) -- compiles against this
//    header and reproduces the reference's run for the same seed (the host
//    draws from the same std::mt19937_64 as the reference, the GPU does the
//    per-site work).
//  * the GPU-resident layer: solve() and the whole-phase calls sweep_all,
//    replica_exchange and icm_all run every replica of the worker in one
//    persistent kernel (pticm_run), the fast path.
// One process drives one GPU: there are no other ranks, so the worker-side
// message handlers (check_icm, check_for_replica_exchange) never receive
// anything.  Errors are thrown as std::runtime_error carrying the C ABI's
// message where the reference asserts or exits.
#pragma once
#include <cstdint>
#include <list>
#include <random>
#include <string>
#include <vector>

#include "pticm.h"

namespace pticm {

typedef std::vector<bool> StateVector;   // include/definitions.hh:76

// include/mpi_defs.hh:12-29
struct Parameters {
    uint64_t seed = 0;
    uint64_t Nt = 20;
    uint64_t pts = 2000;
    uint64_t pre_samples = 2000;
    uint64_t burn_in = 500;
    uint64_t sweeps = 1;
    double T0 = 0.6;
    double T1 = 2.8;
    double cutoff = 0.0;
    double pre_step = 0.1;
    bool inverse = false;
    bool preprocess = false;
    bool log_data = false;
    bool icm = false;
    uint32_t verbosity = 0;
    // GPU engine choices (no reference counterpart)
    uint32_t chains = 2;
    uint32_t exchange = 1;            // 1 even/odd rounds, 0 the reference's shuffled order
    uint32_t best_per_phase = 0;
    uint32_t replicas_per_block = 0;  // 0 automatic
    uint32_t block_threads = 0;       // 0 automatic
    uint32_t icm_algo = 0;            // 0 automatic, 1 BFS, 2 union-find, 3 label propagation
    bool sort_ladder = false;         // sort a --preprocess ladder ascending (ICM on the coldest)
    std::string learned_ladder;       // surrogate network file: learned ladder (multihistogram fallback)
    std::string resume;               // checkpoint to continue from (pticm_checkpoint_load)
    std::string checkpoint;           // checkpoint written after the run (pticm_checkpoint_save)
};

// include/problem.hh:7-98.  The random engine is the reference's: a
// std::mt19937_64 seeded with `seed`, read through a uniform [0, 1)
// distribution (rand_double) or directly (get_rng).
class Problem {
   public:
    Problem() = default;
    Problem(std::string path, uint64_t seed = 0, uint64_t burn_in = UINT64_MAX);
    Problem(double* weights, int* src, int* dest, double* linear, uint64_t seed, uint64_t burn_in, uint64_t N,
            uint64_t M);
    Problem(double* formulation, double* linear, uint64_t seed, uint64_t burn_in, uint64_t N);
    Problem(const Problem&) = delete;
    Problem& operator=(const Problem&) = delete;
    Problem(Problem&& o) noexcept;
    Problem& operator=(Problem&& o) noexcept;
    ~Problem();

    double energy(const StateVector& s) const;
    double energy(bool* s) const;
    double maxcut(const StateVector& s) const;
    double calculate_dE(std::vector<double>& dE, const StateVector& s) const;
    // src/problem.cc:164-181 (on the GPU): dE after site `index` of s flips (s before the flip)
    void incremental_dE(std::vector<double>& dE, const StateVector& s, uint32_t index) const;
    double get_char_scale() const { return info_.char_scale; }
    uint64_t vcount() const { return (uint64_t)info_.n; }
    uint64_t ecount() const { return (uint64_t)info_.m; }
    bool is_sparse() const { return info_.sparse != 0; }
    uint64_t get_burn_in() const { return burn_in_; }
    uint64_t get_seed() const { return seed_; }
    double rand_double() { return unif_(rng_); }
    std::mt19937_64& get_rng() { return rng_; }
    pticm_problem* handle() const { return h_; }

   private:
    void refresh();
    pticm_problem* h_ = nullptr;
    pticm_problem_info info_{};
    uint64_t seed_ = 0, burn_in_ = 0;
    std::mt19937_64 rng_;
    std::uniform_real_distribution<double> unif_{0.0, 1.0};
};

// include/replica.hh:6-66: one replica, held in device memory.  The getters
// return host copies refreshed from the device (get_state() and get_dE()
// return references to them); change a replica through its setters.
// set_state recomputes the fields and energy from the new state (what the
// reference's callers do next with calculate_dE, set_energy and set_dE),
// and set_dE is accepted for the interface: the device keeps the local
// fields of the current state.
class Replica {
   public:
    Replica() = default;
    Replica(Problem& p, double beta, const StateVector& init_state, const std::vector<double>& init_dE,
            double energy, bool log_ene = false, size_t burn_in = 0);
    Replica(const Replica& o);
    Replica(Replica&& o) noexcept;
    Replica& operator=(const Replica& o);
    Replica& operator=(Replica&& o) noexcept;
    ~Replica();

    double get_energy() const { return energy_; }
    void set_energy(double e);
    const StateVector& get_state() const;
    StateVector& get_state();
    uint64_t get_flips() const;
    void set_state(const StateVector& s);
    void set_dE(std::vector<double> dE);
    void set_ene(double e) { set_energy(e); }
    double get_beta() const { return beta_; }
    void set_beta(double beta);
    std::vector<double>& get_dE();
    const StateVector& get_best_state() const;
    size_t get_best_sweep() const;
    double get_best_ene() const;
    const std::list<double>& get_ene_log() const { return ene_log_; }
    // src/replica.cc:5-38: the sequential Metropolis sweep on the GPU with
    // uniforms drawn from p's engine (exactly as many as the reference draws)
    void sweep(Problem& p);
    pticm_replica* handle() const { return h_; }

   private:
    pticm_replica_info info() const;
    pticm_replica* h_ = nullptr;
    const Problem* prob_ = nullptr;
    double energy_ = 0.0, beta_ = 0.0;
    bool log_energy_ = false;
    uint64_t sweeps_ = 0;
    size_t burn_in_ = 0;
    mutable bool state_fresh_ = false, dE_fresh_ = false, best_fresh_ = false;
    mutable StateVector state_, best_state_;
    mutable std::vector<double> dE_;
    std::list<double> ene_log_;
    std::vector<double> u_, elog_;
};

// include/mpi_defs.hh:33-65.  One worker holds every replica (wid 0 of one).
// The manager's fields keep the reference's names; the per-replica layer
// (initialize_replicas, try_replica_exchange, icm) uses them, while ctx is
// the GPU-resident run of solve() and the whole-phase calls.
struct PTWorker {
    int wid = 0;
    int numw = 1;
    uint64_t worker_r = 0, last_r = 0, loc_r = 0;
    Parameters params;
    Problem p;
    std::vector<double> beta_values;          // 2*Nt (two chains)
    uint64_t swaps = 0;
    uint32_t Nc = 0;
    double characteristic_scale = 0.0;
    std::vector<double> energy_values_global; // 2*Nt, gathered after the sweeps
    std::vector<uint32_t> chain_1_exchange_order;
    std::vector<uint32_t> chain_2_exchange_order;
    std::vector<uint8_t> chain_index_global;
    uint32_t exchange_index = 0;
    std::vector<uint32_t> beta_indices;       // slot -> replica
    std::vector<int> replica_workers;         // replica -> rank (all 0)
    std::vector<uint32_t> swap_attempts;      // per slot
    std::vector<uint32_t> swap_successes;
    std::vector<uint8_t> chain_index_local;   // replica -> chain
    std::vector<double> energy_values_local;  // replica -> energy after the sweeps
    std::vector<double> beta_values_local;    // replica -> beta
    std::vector<Replica> replicas;
    pticm_ctx* ctx = nullptr;
    PTWorker() = default;
    PTWorker(const PTWorker&) = delete;
    PTWorker& operator=(const PTWorker&) = delete;
    ~PTWorker();
};

// include/solver.hh:6 -- the whole PT-ICM run on the GPU-resident layer,
// printing the reference's report
void solve(PTWorker& w, std::string& problem_path, double& best_ene, size_t& flips, StateVector& best_state);

// The folder mode of src/main.cc:149-207 (unreachable there: its parser never
// sets the folder): every problem file of `folder`, `restarts` runs each, one
// CSV row per run with the reference's columns.  All runs with ladders of one
// length share one batched launch; returns the rows written.
size_t solve_folder(PTWorker& w, const std::string& folder, const std::string& csv_path, size_t restarts);

// src/utils.cc:6-22
void beta_linspace(double* temps, double T0, double T1, uint64_t num_temp, bool inverse);

// include/utils.hh:91-93 (src/cae_estimator.cc:295-428): fills w.beta_values
// with the multihistogram constant-acceptance ladder and sets w.params.Nt
void get_beta(PTWorker& w, double estep, double step_size, double r, size_t num_samples);

// The ladder of src/initialization.cc:103-157 (linspace, --preprocess, or the
// learned ladder) into w.beta_values, w.params.Nt set to its length
void choose_ladder(PTWorker& w);

// include/initialization.hh:6-10 (src/initialization.cc:5-191)
void read_problem(PTWorker& w, std::string problem_path);
void initialize_temperatures(PTWorker& w);    // ladder, Nc, replica chains; creates the GPU-resident run
void initialize_replicas(PTWorker& w);        // Bernoulli(1/2) states from w.p's engine, one Replica each
void initialize_replica_exchanges(PTWorker& w);

// include/replica_exchange.hh:6-12 (src/replica_exchange.cc:5-125): one
// attempt of chain `chain_index` at the next pair of the shared order
void try_replica_exchange(PTWorker& w, uint8_t chain_index);
void do_replica_exchange_local(PTWorker& w, double beta_old, double beta_new, uint8_t chain_index);
void check_for_replica_exchange(PTWorker& w);

// include/icm.hh:6-15 (src/icm.cc:8-215): the cluster move of the pair at
// temperature slot `target_replica`; the overlap and the cluster are
// computed on the GPU
void check_icm(PTWorker& w);
void icm(PTWorker& w, size_t target_replica);
void bfs_icm(Problem& p, int64_t seed_val, bool* state_1, bool* state_2);
int64_t xor_icm(PTWorker& w, bool* state_1, bool* state_2);

// include/mpi_utils.hh:6-18 (src/mpi_utils.cc:77-226)
void gather_energy_values(PTWorker& w);
Replica& get_replica(PTWorker& w, double beta, uint8_t chain);
// The best (energy, sweep, state) and the flip count over w.replicas when
// the worker holds Replica objects, else over the GPU-resident run
void gather_best_energy_values(PTWorker& w, double& best_ene, size_t& best_sweep, StateVector& best_state);
uint64_t get_flips(PTWorker& w);

// One phase of the PT step for every replica of the GPU-resident run
// (src/solver.cc:69-106 as whole phases): Replica::sweep x sweeps, the Nt-1
// exchange attempts per chain, the Nc ICMs.
void sweep_all(PTWorker& w);
void replica_exchange(PTWorker& w);
void icm_all(PTWorker& w);

}  // namespace pticm
