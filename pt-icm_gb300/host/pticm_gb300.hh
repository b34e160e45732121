// pticm_gb300.hh -- the reference's C++ interface (libreplica headers
// problem.hh / replica_exchange.hh / icm.hh / solver.hh / utils.hh / mpi_defs.hh)
// over the GB300 engine's C ABI (include/pticm.h).
//
// Code written against the reference keeps compiling: the same names,
// argument meanings and results.  Differences of shape follow from the GPU
// design: all replicas of a run live on the GPU inside a PTWorker, so the
// per-replica `Replica::sweep` and per-attempt `try_replica_exchange` become
// whole-phase calls (every replica swept / every pair attempted), and errors
// are thrown as std::runtime_error carrying the C ABI's message where the
// reference asserts or exits.
#pragma once
#include <cstdint>
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

// include/problem.hh:7-98
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
    double maxcut(const StateVector& s) const;
    double calculate_dE(std::vector<double>& dE, const StateVector& s) const;
    double get_char_scale() const { return info_.char_scale; }
    uint64_t vcount() const { return (uint64_t)info_.n; }
    uint64_t ecount() const { return (uint64_t)info_.m; }
    bool is_sparse() const { return info_.sparse != 0; }
    uint64_t get_burn_in() const { return burn_in_; }
    uint64_t get_seed() const { return seed_; }
    pticm_problem* handle() const { return h_; }

   private:
    void refresh();
    pticm_problem* h_ = nullptr;
    pticm_problem_info info_{};
    uint64_t seed_ = 0, burn_in_ = 0;
};

// include/mpi_defs.hh:33-65: the state solve() drives.  On the GPU one
// worker holds every replica; the fields below mirror the manager's view.
struct PTWorker {
    int wid = 0;
    int numw = 1;
    Parameters params;
    Problem p;
    std::vector<double> beta_values;        // 2*Nt (two chains)
    std::vector<uint32_t> beta_indices;     // slot -> replica
    std::vector<uint32_t> swap_attempts;    // per slot
    std::vector<uint32_t> swap_successes;
    uint64_t swaps = 0;
    uint32_t Nc = 0;
    double characteristic_scale = 0.0;
    pticm_ctx* ctx = nullptr;
    PTWorker() = default;
    PTWorker(const PTWorker&) = delete;
    PTWorker& operator=(const PTWorker&) = delete;
    ~PTWorker();
};

// include/solver.hh:6 -- the whole PT-ICM run, printing the reference's report
void solve(PTWorker& w, std::string& problem_path, double& best_ene, size_t& flips, StateVector& best_state);

// The folder mode of src/main.cc:149-207 (unreachable there: its parser never
// sets the folder): every problem file of `folder`, `restarts` runs each, one
// CSV row per run with the reference's columns.  All runs with ladders of one
// length share one batched launch; returns the rows written.
size_t solve_folder(PTWorker& w, const std::string& folder, const std::string& csv_path, size_t restarts);

// src/mpi_utils.cc:6-22
void beta_linspace(double* temps, double T0, double T1, uint64_t num_temp, bool inverse);

// include/utils.hh:91-93 (src/cae_estimator.cc:295-428): fills w.beta_values
// with the multihistogram constant-acceptance ladder and sets w.params.Nt
void get_beta(PTWorker& w, double estep, double step_size, double r, size_t num_samples);

// The ladder of src/initialization.cc:103-157 (linspace, --preprocess, or the
// learned ladder) into w.beta_values, w.params.Nt set to its length
void choose_ladder(PTWorker& w);

// src/initialization.cc:103-191 / 63-100: ladder, Nc, replicas, exchange state
void initialize_temperatures(PTWorker& w);
void initialize_replicas(PTWorker& w);

// One phase of the PT step for every replica (src/solver.cc:69-106):
// Replica::sweep x sweeps, the Nt-1 exchange attempts per chain, the Nc ICMs.
void sweep_all(PTWorker& w);
void replica_exchange(PTWorker& w);
void icm_all(PTWorker& w);

// src/mpi_utils.cc:103-176
void gather_best_energy_values(PTWorker& w, double& best_ene, size_t& best_sweep, StateVector& best_state);
uint64_t get_flips(PTWorker& w);

}  // namespace pticm
