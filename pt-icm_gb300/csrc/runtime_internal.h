// runtime_internal.h -- host-side launch planning shared by the context API
// (runtime.cu) and the allocation-free entry point (noalloc.cu).
#pragma once
#include <cuda_runtime.h>

#include <limits>
#include <string>
#include <vector>

#include "pticm.h"
#include "pticm_engine.h"
#include "problem_host.h"

namespace pticm {

constexpr long long kNoBest = std::numeric_limits<long long>::max();

template <typename T>
struct DArr {
    T* p = nullptr;
    size_t n = 0;
    DArr() = default;
    DArr(const DArr&) = delete;
    DArr& operator=(const DArr&) = delete;
    ~DArr() { release(); }
    void release() {
        if (p) cudaFree(p);
        p = nullptr;
        n = 0;
    }
    cudaError_t alloc(size_t count) {
        release();
        n = count;
        if (count == 0) return cudaSuccess;
        cudaError_t e = cudaMalloc(&p, count * sizeof(T));
        if (e != cudaSuccess) { p = nullptr; n = 0; return e; }
        return cudaMemset(p, 0, count * sizeof(T));
    }
    cudaError_t upload(const std::vector<T>& v, size_t extra = 0) {
        cudaError_t e = alloc(v.size() + extra);
        if (e != cudaSuccess || v.empty()) return e;
        return cudaMemcpy(p, v.data(), v.size() * sizeof(T), cudaMemcpyHostToDevice);
    }
    cudaError_t download(std::vector<T>& v) const {
        v.resize(n);
        if (!n) return cudaSuccess;
        return cudaMemcpy(v.data(), p, n * sizeof(T), cudaMemcpyDeviceToHost);
    }
};

inline uint32_t align16(uint64_t x) { return (uint32_t)((x + 15) & ~15ull); }

inline int32_t pad16(int64_t n) { return (int32_t)((n + 15) & ~15ll); }

struct LaunchConfig {
    int rpc = 0, group = 0, threads = 0, teams = 1;
    bool block_team = false;
    bool narrow = false;         // block team on the narrow-bound kernel (kNarrowThreads, 120 registers)
    bool state_global = false;   // replica state and ICM scratch in device memory
    bool field_gather = false;   // spins in shared memory, fields gathered at each visit
    SmemPlan plan{};
};

// Shared-memory needs of the instances of one launch (region-wise maxima).
struct PlanDims {
    uint64_t n_stage = 0, nnz_stage = 0, ncolors = 0, n_h = 0, spin_sites = 0, nt_kst = 0, R = 0, rpc = 0, nt = 0,
             chains_m = 0, icm_bytes = 0, max_n_pad = 0, max_kmax = 0;
    int teams = 0;
    bool stage = false, replay = false, state_global = false, field_gather = false, icm_split = false;
    void add(const InstanceDesc& D, bool stage_this, int teams_of_instance);
};
SmemPlan layout_plan(const PlanDims& d);
SmemPlan make_plan(const InstanceDesc& D, bool replay, int teams, int threads, bool stage_adj,
                   bool state_global = false, bool field_gather = false, bool icm_split = false);
constexpr uint32_t kSmemLimit = 232448 - 1024;   // 227 KB opt-in per block, less static smem

int choose_config(const HostProblem& P, const pticm_opts& o, bool replay, InstanceDesc& D, LaunchConfig& cfg,
                  std::string& msg);
int engine_flags(const HostProblem& P, const pticm_opts& o);
// Schedule of a launch that holds one instance: block b runs rank b.
void single_instance_schedule(int group, std::vector<int32_t>& sched_off, std::vector<int32_t>& sched);
// Per-instance engine choices of a configured instance: cluster search and
// adjacency staging.
void finish_desc(InstanceDesc& D, const HostProblem& P, const pticm_opts& o, const LaunchConfig& cfg);
int ladder_tables(const HostProblem& P, const double* beta, int nt, int nc_req, bool icm, int chains,
                  std::vector<uint32_t>& thr, std::vector<double>& ptab);

// One multihistogram input in make_histogram's layout
// (src/cae_estimator.cc:45-69) and its solution.
struct MhInput {
    std::vector<uint32_t> hist;
    std::vector<uint64_t> hoff, hlen;
    std::vector<double> emin, beta;
    double estep = 2.0;
    uint64_t n = 0;
    double max_emax = 0.0;
};
struct MhOutput {
    std::vector<double> logdos, logZ;
    double min_emin = 0.0;
    uint64_t iters = 0;
};
constexpr long long kMhistMaxIters = 300000;
int mhist_dos_multi(const std::vector<const MhInput*>& in, std::vector<MhOutput>& out);
int compact_slot_hist(const unsigned* rows, int nt, int chains, long long nbins, long long lo, const double* hb,
                      double estep, MhInput& I);
int mhist_dos_impl(const uint32_t* hist, const uint64_t* hoff, const uint64_t* hlen, uint32_t nt,
                   const double* beta, const double* emin, double estep, uint64_t n, double max_emax,
                   std::vector<double>& logdos, std::vector<double>& logZ, double& min_emin, uint64_t& iters);
int slot_hist_dos(const unsigned* rows, int nt, int chains, long long nbins, long long lo, const double* hb,
                  double estep, std::vector<double>& dos, std::vector<double>& logZ, double& min_emin,
                  uint64_t& iters);
// energy range of a problem: every energy lies in [-W, W] with the parity of W
long long energy_bound(const HostProblem& P);

const HostProblem& problem_host(const pticm_problem* p);
// The device copy of a problem in the engine's site order (uploaded on first
// use and kept with the problem): CSR rows, packed adjacency (col << 8 |
// uint8 J), linear terms, perm (device -> original site) and iperm
// (original -> device site).
struct ProblemDevice {
    const int32_t* row;
    const uint32_t* adj;
    const int32_t* h;
    const int32_t* perm;
    const int32_t* iperm;
    int n, n_pad, kmax;
    bool has_h;
};
int problem_device(const pticm_problem* p, ProblemDevice* out);
void set_last_error(const std::string& m);

cudaError_t launch_engine(const EngineArgs& A, int threads, bool replay, bool block_team, bool narrow,
                          bool cooperative, cudaStream_t stream);
cudaError_t engine_max_blocks_per_sm(bool replay, bool block_team, bool narrow, int threads, size_t smem, int* out);
cudaError_t launch_load_states(const uint8_t* src, const int32_t* iperm, int8_t* spins, int R, int n, int n_pad,
                               cudaStream_t stream);
cudaError_t launch_init_spins(const EngineArgs& A, const int32_t* rep_inst, int total_reps,
                              unsigned long long seed, cudaStream_t stream);
cudaError_t launch_recompute(const EngineArgs& A, const int32_t* rep_inst, int total_reps, int write_back,
                             unsigned long long* mismatches, long long* E_out, long long* cut2_out,
                             cudaStream_t stream);

}  // namespace pticm
