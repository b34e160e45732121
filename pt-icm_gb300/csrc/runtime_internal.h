// runtime_internal.h -- host-side launch planning shared by the context API
// (runtime.cu) and the allocation-free entry point (noalloc.cu).
#pragma once
#include <cuda_runtime.h>

#include <string>
#include <vector>

#include "pticm.h"
#include "pticm_engine.h"
#include "problem_host.h"

namespace pticm {

struct LaunchConfig {
    int rpc = 0, group = 0, threads = 0, teams = 1;
    bool block_team = false;
    SmemPlan plan{};
};

SmemPlan make_plan(const InstanceDesc& D, bool replay, int teams, int threads, bool stage_adj);
int choose_config(const HostProblem& P, const pticm_opts& o, bool replay, InstanceDesc& D, LaunchConfig& cfg,
                  std::string& msg);
int engine_flags(const HostProblem& P, const pticm_opts& o);
int ladder_tables(const HostProblem& P, const double* beta, int nt, int nc_req, bool icm, int chains,
                  std::vector<uint32_t>& thr, std::vector<double>& ptab);

const HostProblem& problem_host(const pticm_problem* p);
void set_last_error(const std::string& m);

cudaError_t launch_engine(const EngineArgs& A, int threads, bool replay, bool block_team, bool cooperative,
                          cudaStream_t stream);
cudaError_t engine_max_blocks_per_sm(bool replay, bool block_team, int threads, size_t smem, int* out);
cudaError_t launch_recompute(const EngineArgs& A, const int32_t* rep_inst, int total_reps, int write_back,
                             unsigned long long* mismatches, long long* E_out, long long* cut2_out,
                             cudaStream_t stream);

}  // namespace pticm
