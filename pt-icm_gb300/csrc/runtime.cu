// runtime.cu -- host runtime and C ABI of the PT-ICM engine (include/pticm.h).
//
// A pticm_ctx is the GPU-resident equivalent of the reference's PTWorker
// (include/mpi_defs.hh:33-65) for one problem: every replica, the
// temperature ladder, the slot->replica map (beta_indices), exchange
// statistics and best-state tracking live in device memory; the host only
// launches the engine and reads results back.
#include <cuda_runtime.h>

#include <algorithm>
#include <cfloat>
#include <cmath>
#include <cstring>
#include <limits>
#include <memory>
#include <random>
#include <string>
#include <vector>

#include "pticm.h"
#include "pticm_device.cuh"
#include "pticm_engine.h"
#include "problem_host.h"
#include "runtime_internal.h"
#include "mhist_host.h"
#include "mhist_job.h"

namespace pticm {
cudaError_t launch_recompute(const EngineArgs& A, const int32_t* rep_inst, int total_reps, int write_back,
                             unsigned long long* mismatches, long long* E_out, long long* cut2_out,
                             cudaStream_t stream);
cudaError_t launch_init_spins(const EngineArgs& A, const int32_t* rep_inst, int total_reps,
                              unsigned long long seed, cudaStream_t stream);
cudaError_t launch_evaluate(const int32_t* row, const uint32_t* adj, const int32_t* h, int n, int n_pad,
                            const int8_t* states, int count, long long* E_out, long long* cut2_out,
                            int32_t* dE_out, cudaStream_t stream);
cudaError_t launch_philox_probe(const uint4* ctr, const uint2* key, uint4* out, int count, cudaStream_t stream);
}  // namespace pticm

using namespace pticm;

namespace {

thread_local std::string g_err;

int fail(int code, const std::string& m) {
    g_err = m;
    return code;
}

#define CK(x)                                                                                    \
    do {                                                                                         \
        cudaError_t e_ = (x);                                                                    \
        if (e_ != cudaSuccess) return fail(PTICM_ERR_CUDA, std::string(#x) + ": " + cudaGetErrorString(e_)); \
    } while (0)

int check_device() {
    int count = 0;
    cudaError_t e = cudaGetDeviceCount(&count);
    if (e != cudaSuccess || count == 0)
        return fail(PTICM_ERR_NODEVICE, "no CUDA device is available; the PT-ICM engine has no CPU path");
    return PTICM_OK;
}

}  // namespace

struct pticm_problem {
    HostProblem hp;
    // device copy for pticm_problem_evaluate and the single-replica calls
    DArr<int32_t> d_row, d_h, d_perm, d_iperm;
    DArr<uint32_t> d_adj;
    bool uploaded = false;
};

struct pticm_ctx {
    HostProblem P;
    pticm_opts o{};
    int nt = 0, C = 2, R = 0, nc = 0;
    bool ladder_set = false, states_set = false;
    std::vector<double> beta;
    InstanceDesc desc{};
    int rpc = 0, group = 0, threads = 0, teams = 1;
    bool block_team = false, narrow = false;
    SmemPlan plan{};
    uint64_t steps_done = 0, attempts = 0;
    double last_ms = 0.0;
    cudaStream_t stream = nullptr;
    cudaEvent_t ev0 = nullptr, ev1 = nullptr;
    // device pools
    DArr<InstanceDesc> d_desc;
    DArr<int32_t> d_sched_off, d_sched, d_rep_inst, d_row, d_col, d_h, d_perm;
    DArr<uint32_t> d_adj, d_thr, d_slot, d_order, d_cursor;
    DArr<double> d_beta, d_ptab;
    DArr<int8_t> d_spins, d_pub, d_best_state;
    DArr<int32_t> d_fields;
    DArr<long long> d_E, d_Epub, d_bestE;
    DArr<unsigned long long> d_flips, d_bestSweep, d_att, d_succ, d_mismatch, d_prof;
    bool profiling = false;
    DArr<unsigned int> d_hist;   // pilot energy histograms (multihistogram ladder)
    DArr<long long> d_obs, d_mag_pub;   // magnetisation sums per slot, published magnetisations
    long long hist_lo = 0, hist_nbins = 0;
    uint64_t hist_from = 0;
    DArr<unsigned int> d_bar;
    DArr<int> d_abort;
    DArr<DevStatus> d_status;
    DArr<uint8_t> d_states_in;  // caller states in the original site order (pticm_set_states)
    DArr<uint8_t> d_icm_pool;   // ICM scratch when the replicas live in device memory
    long long icm_stride = 0;
    long long ebound = -1;      // energy_bound(P), once
    DArr<long long> d_icm_force;   // per-pair seeds of pticm_icm_pairs
    // bounded waits: limit (0 = kWaitLimitNs) and the barrier test hook
    unsigned long long wait_limit_ns = 0;
    int bar_phantom = 0;
    // the inputs of the last launch configuration (it depends on nothing else
    // once the context exists): replay, ICM pairs, histogram rows
    bool configured = false;
    bool cfg_replay = false;
    int32_t cfg_nc = -1;
    int64_t cfg_hist_off = 0, cfg_hist_lo = 0, cfg_hist_nbins = 0;

    ~pticm_ctx() {
        if (ev0) cudaEventDestroy(ev0);
        if (ev1) cudaEventDestroy(ev1);
        if (stream) cudaStreamDestroy(stream);
    }
};

namespace pticm {

void PlanDims::add(const InstanceDesc& D, bool stage_this, int teams_of_instance) {
    const uint64_t kst = (uint64_t)D.kmax + 1, m = (uint64_t)std::max(D.nt - 1, 1);
    if (stage_this) {
        stage = true;
        n_stage = std::max(n_stage, (uint64_t)D.n);
        nnz_stage = std::max(nnz_stage, (uint64_t)D.nnz);
    }
    ncolors = std::max(ncolors, (uint64_t)D.ncolors);
    if (D.has_h) n_h = std::max(n_h, (uint64_t)D.n);
    spin_sites = std::max(spin_sites, (uint64_t)D.rpc * (uint64_t)D.n_pad);
    nt_kst = std::max(nt_kst, (uint64_t)D.nt * kst);
    R = std::max(R, (uint64_t)D.R);
    rpc = std::max(rpc, (uint64_t)D.rpc);
    nt = std::max(nt, (uint64_t)D.nt);
    chains_m = std::max(chains_m, (uint64_t)D.chains * m);
    icm_bytes = std::max(icm_bytes, icm_block_bytes(teams_of_instance, D.n_pad));
    teams = std::max(teams, teams_of_instance);
    max_n_pad = std::max(max_n_pad, (uint64_t)D.n_pad);
    max_kmax = std::max(max_kmax, (uint64_t)D.kmax);
}

// Shared-memory layout for a launch; every region starts on 16 bytes and is
// the largest any instance of the launch needs.
SmemPlan layout_plan(const PlanDims& d) {
    SmemPlan S{};
    uint64_t off = 0;
    auto take = [&](uint64_t bytes) {
        const uint32_t o = (uint32_t)off;
        off = align16(off + bytes);
        return o;
    };
    S.mbar = take(16);
    S.stage_adj = d.stage ? 1 : 0;
    if (d.stage) {
        S.row = take(align16((d.n_stage + 1) * 4));
        S.adj = take(align16(d.nnz_stage * 4));
    }
    S.col = take((d.ncolors + 1) * 4);
    S.h = take(d.n_h * 4);
    S.state_global = d.state_global ? 1 : 0;
    S.field_gather = d.field_gather ? 1 : 0;
    S.spin = take(d.state_global ? 0 : d.spin_sites);
    S.field = take((d.state_global || d.field_gather) ? 0 : d.spin_sites * 4);
    S.thr = take(d.field_gather ? 0 : d.nt_kst * 4);
    S.ptab = take(d.replay ? d.nt_kst * 8 : 0);
    S.slot = take(d.R * 4);
    S.rslot = take(d.rpc * 8);
    S.order = take(d.nt * 4);
    S.beta = take(d.nt * 8);
    S.dbeta = take(d.nt * 8);
    S.E = take(d.R * 8);
    S.dEp = take(d.rpc * 4);
    S.flp = take(d.rpc * 4);
    S.bestE = take(d.rpc * 8);
    S.flips = take(d.rpc * 8);
    S.improved = take(d.rpc * 4);
    S.att = take(d.R * 4);
    S.succ = take(d.R * 4);
    S.xlogu = take(d.chains_m * 4 + 16);
    S.xrand = take(d.chains_m * 4 + 16);
    S.xlevel = take(d.nt * 4);
    S.xpos = take(d.nt * 4);
    S.icm_team_bytes = icm_team_bytes((int32_t)d.max_n_pad);
    S.teams = d.teams;
    S.icm_split = d.icm_split ? 1 : 0;
    S.icm = take(d.icm_split ? (uint64_t)icm_team_bytes((int32_t)d.max_n_pad)
                             : ((d.state_global || d.field_gather) ? 0 : d.icm_bytes));
    S.mag = take(d.rpc * 8);
    S.misc = take(64 + 8 * 32 + 4 * 64 + 64);
    S.total = (uint32_t)off;
    S.max_n_pad = (int32_t)d.max_n_pad;
    S.max_kmax = (int32_t)d.max_kmax;
    S.max_R = (int32_t)d.R;
    S.max_nt = (int32_t)d.nt;
    return S;
}

SmemPlan make_plan(const InstanceDesc& D, bool replay, int teams, int threads, bool stage_adj, bool state_global,
                   bool field_gather, bool icm_split) {
    PlanDims d;
    d.replay = replay;
    d.state_global = state_global;
    d.field_gather = field_gather;
    d.icm_split = field_gather && icm_split && teams == 1;
    d.add(D, stage_adj, teams);
    (void)threads;
    return layout_plan(d);
}

// Choose replicas per block, block size, ICM teams and the smem plan for an
// instance described by D (D.rpc / D.group are filled in).  Allocates
// nothing: it only queries device attributes and occupancy.
int choose_config(const HostProblem& P, const pticm_opts& o, bool replay, InstanceDesc& D, LaunchConfig& cfg,
                  std::string& msg) {
    const int R = D.R, n = (int)P.n;
    const int npairs = D.nc * (D.chains / 2);
    int max_class = 1;
    for (int k = 0; k < P.ncolors; k++) max_class = std::max(max_class, P.color_off[k + 1] - P.color_off[k]);
    auto fits = [&](int rpc, int threads, int teams, bool stage, SmemPlan& out) {
        InstanceDesc t = D;
        t.rpc = rpc;
        t.group = R / rpc;
        out = make_plan(t, replay, teams, threads, stage);
        return out.total <= kSmemLimit;
    };
    int rpc = (int)o.replicas_per_block;
    if (replay) rpc = R;
    int dev = 0, sms = 0;
    cudaError_t e = cudaGetDevice(&dev);
    if (e == cudaSuccess) e = cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
    if (e != cudaSuccess) { msg = cudaGetErrorString(e); return PTICM_ERR_CUDA; }
    if (rpc <= 0) {
        // one replica per block (one SM each) while the replicas fit on the
        // GPU at once; otherwise the smallest divisor of R that does
        rpc = 1;
        while (rpc < R && (R / rpc > sms || R % rpc != 0)) rpc++;
    }
    if (rpc <= 0 || R % rpc != 0) { msg = "replicas_per_block must divide the replica count"; return PTICM_ERR_INVALID; }
    int group = R / rpc;
    int threads = (int)o.block_threads;
    if (replay) threads = std::min(1024, 32 * std::max(1, std::min(R, 32)));
    if (threads <= 0) {
        // several replicas per block: the 512-thread bound; one replica per
        // block: at most the narrow-bound block (on N=2000, 512 threads at
        // 120 registers beat 1024 threads at 64 by 11 %)
        if (rpc > 1) threads = kNarrowThreads;
        else threads = std::min(kNarrowThreads, std::max(128, ((std::max(max_class, n / 2) + 31) / 32) * 32));
    }
    if (threads % 32 != 0 || threads > 1024) {
        msg = "block_threads must be a multiple of 32, at most 1024";
        return PTICM_ERR_INVALID;
    }
    if (!replay && rpc > 1 && threads > kNarrowThreads) {
        msg = "block_threads must be at most 512 with several replicas per block";
        return PTICM_ERR_INVALID;
    }
    bool block_team = (rpc == 1) && !replay;
    // ICM teams: one warp per pair on small instances; from 768 sites on the
    // whole block is one team (pairs in sequence), which is faster per pair
    int teams = (block_team || D.n_pad >= 768) ? 1 : std::max(1, std::min(threads / 32, std::max(1, npairs)));
    SmemPlan plan;
    bool stage = true, global = false;
    const int teams0 = teams;
    while (!fits(rpc, threads, teams, stage, plan)) {
        if (stage) { stage = false; continue; }
        if (teams > 1) { teams = std::max(1, teams / 2); continue; }
        // the replicas do not fit shared memory: keep them (and the ICM
        // scratch) in device memory, where the 129 MB L2 holds them
        if (replay) {
            msg = "replay needs the replicas in shared memory; the instance is too large";
            return PTICM_ERR_UNSUPPORTED;
        }
        // first choice: the spins alone in shared memory, fields gathered
        // at each visit (no field atomics).  Several replicas per block
        // (each neighbour-list read serves all of them, and the cluster
        // search's scratch fits in shared memory beside their spins) while
        // the blocks still cover most SMs: on N=20000, R=512, four replicas
        // in each of 128 blocks measured 11.1 G attempts/s against 8.7 G
        // with one replica in each of 512 blocks.  Otherwise one replica per
        // block, the largest block that keeps all R blocks resident.
        auto gather_multi = [&](int rp) {
            if (rp < 2 || R % rp != 0 || o.block_threads > (uint32_t)kNarrowThreads) return false;
            const int t = o.block_threads ? (int)o.block_threads : kNarrowThreads;
            InstanceDesc d1 = D;
            d1.rpc = rp;
            d1.group = R / rp;
            for (bool split : {true, false}) {
                const SmemPlan p1 = make_plan(d1, false, 1, t, false, false, true, split);
                int per_sm = 0;
                if (p1.total > kSmemLimit ||
                    engine_max_blocks_per_sm(false, false, false, t, p1.total, &per_sm) != cudaSuccess ||
                    (int64_t)per_sm * sms < R / rp)
                    continue;
                rpc = rp;
                threads = t;
                block_team = false;
                teams = 1;
                plan = p1;
                return true;
            }
            return false;
        };
        auto gather_one = [&]() {
            const int sizes[4] = {1024, 512, 256, 128};
            const int asked[1] = {(int)o.block_threads};
            const int* cand = o.block_threads ? asked : sizes;
            const int ncand = o.block_threads ? 1 : 4;
            for (int ci = 0; ci < ncand; ci++) {
                const int t = cand[ci];
                InstanceDesc d1 = D;
                d1.rpc = 1;
                d1.group = R;
                const SmemPlan p1 = make_plan(d1, false, 1, t, false, false, true);
                if (p1.total > kSmemLimit) continue;
                int per_sm = 0;
                if (engine_max_blocks_per_sm(false, true, false, t, p1.total, &per_sm) != cudaSuccess) continue;
                if ((int64_t)per_sm * sms < R) continue;
                rpc = 1;
                threads = t;
                block_team = true;
                teams = 1;
                plan = p1;
                return true;
            }
            return false;
        };
        bool gathered = false;
        if (o.replicas_per_block == 0) {
            for (int rp : {4, 2})
                if (!gathered && R / rp >= (3 * sms) / 4) gathered = gather_multi(rp);
            if (!gathered) gathered = gather_one();
        } else if (o.replicas_per_block == 1) {
            gathered = gather_one();
        } else {
            gathered = gather_multi((int)o.replicas_per_block);
        }
        if (gathered) {
            cfg.field_gather = true;
            break;
        }
        global = true;
        // with the state in device memory a block needs little shared
        // memory: one replica per block (the whole block is one ICM team)
        // when smaller blocks let all R blocks be resident at once
        bool placed = false;
        if (o.replicas_per_block == 0 && o.block_threads == 0) {
            for (int t : {512, 256, 128}) {
                InstanceDesc d1 = D;
                d1.rpc = 1;
                d1.group = R;
                const SmemPlan p1 = make_plan(d1, false, 1, t, false, true);
                if (p1.total > kSmemLimit) continue;
                int per_sm = 0;
                if (engine_max_blocks_per_sm(false, true, false, t, p1.total, &per_sm) != cudaSuccess) continue;
                if ((int64_t)per_sm * sms < R) continue;
                rpc = 1;
                threads = t;
                block_team = true;
                teams = 1;
                plan = p1;
                placed = true;
                break;
            }
        }
        if (!placed) {
            InstanceDesc t = D;
            t.rpc = rpc;
            t.group = R / rpc;
            teams = block_team ? 1 : std::min(teams0, 16);
            plan = make_plan(t, false, teams, threads, false, true);
        }
        if (plan.total > kSmemLimit) {
            msg = "the per-temperature tables of the instance do not fit in shared memory";
            return PTICM_ERR_UNSUPPORTED;
        }
        break;
    }
    cfg.state_global = global;
    group = R / rpc;
    // a block team takes the narrow-bound kernel when its blocks stay
    // resident with one block per SM
    bool narrow = false;
    if (block_team && threads <= kNarrowThreads) {
        int per_sm = 0;
        if (engine_max_blocks_per_sm(false, true, true, threads, plan.total, &per_sm) == cudaSuccess &&
            (int64_t)per_sm * sms >= group)
            narrow = true;
    }
    cfg.narrow = narrow;
    D.rpc = rpc;
    D.group = group;
    D.teams = teams;
    cfg.rpc = rpc;
    cfg.group = group;
    cfg.threads = threads;
    cfg.teams = teams;
    cfg.block_team = block_team;
    cfg.plan = plan;
    if (group > 1) {
        int per_sm = 0;
        e = engine_max_blocks_per_sm(replay, block_team, narrow, threads, plan.total, &per_sm);
        if (e != cudaSuccess) { msg = cudaGetErrorString(e); return PTICM_ERR_CUDA; }
        if ((int64_t)per_sm * sms < group) {
            msg = "the replica blocks of one instance cannot all be resident (" + std::to_string(group) +
                  " blocks, " + std::to_string(per_sm * sms) + " resident); raise replicas_per_block";
            return PTICM_ERR_UNSUPPORTED;
        }
    }
    return PTICM_OK;
}

// Engine flags for the options: exchange order, best tracking, cluster search
// (automatic: union-find with Afforest sampling, the fastest measured on
// sparse and dense graphs alike; BFS and label propagation on request).
int engine_flags(const HostProblem& P, const pticm_opts& o) {
    (void)P;
    int algo = ENGINE_ICM_UNION_FIND;
    if (o.icm_algo == 1) algo = ENGINE_ICM_BFS;
    else if (o.icm_algo == 2) algo = ENGINE_ICM_UNION_FIND;
    else if (o.icm_algo == 3) algo = ENGINE_ICM_LABEL_PROP;
    return (o.best_per_phase ? ENGINE_BEST_PER_PHASE : 0) | (o.exchange == 1 ? ENGINE_EXCHANGE_EVEN_ODD : 0) | algo;
}

long long energy_bound(const HostProblem& P) {
    long long directed = 0, lin = 0;
    for (int64_t i = 0; i < P.n; i++) {
        lin += std::llabs((long long)P.h[i]);
        for (int64_t a = P.row[i]; a < P.row[i + 1]; a++) directed += std::llabs((long long)P.w[a]);
    }
    return directed / 2 + lin;
}

void single_instance_schedule(int group, std::vector<int32_t>& sched_off, std::vector<int32_t>& sched) {
    sched_off.resize((size_t)group + 1);
    sched.resize(2 * (size_t)group);
    for (int b = 0; b <= group; b++) sched_off[b] = b;
    for (int b = 0; b < group; b++) {
        sched[2 * b] = 0;
        sched[2 * b + 1] = b;
    }
}

void finish_desc(InstanceDesc& D, const HostProblem& P, const pticm_opts& o, const LaunchConfig& cfg) {
    D.icm_algo = engine_flags(P, o) & ENGINE_ICM_MASK;
    D.stage = cfg.plan.stage_adj;
    D.rpc = cfg.rpc;
    D.group = cfg.group;
}

// Acceptance tables of a ladder: thr = ceil(exp(-beta*dE) 2^32) (all-ones:
// always) and the FP64 exp(-beta*dE) itself, dE = 2t, t = 1..kmax; and the
// ICM pair count of src/initialization.cc:158-164 (nc < 0) or nc.
int ladder_tables(const HostProblem& P, const double* beta, int nt, int nc_req, bool icm, int chains,
                  std::vector<uint32_t>& thr, std::vector<double>& ptab) {
    const int kst = P.kmax + 1;
    thr.assign((size_t)nt * kst, 0xFFFFFFFFu);
    ptab.assign((size_t)nt * kst, 1.0);
    for (int k = 0; k < nt; k++)
        for (int t = 1; t < kst; t++) {
            const double dE = 2.0 * t;
            const double p = std::exp(-beta[k] * dE);   // the reference's expression, src/replica.cc:35
            ptab[(size_t)k * kst + t] = p;
            const double scaled = std::ceil(p * 4294967296.0);
            thr[(size_t)k * kst + t] = (p >= 1.0 || scaled >= 4294967295.0) ? 0xFFFFFFFFu : (uint32_t)scaled;
        }
    int count = 0;
    if (nc_req >= 0) {
        count = std::min(nc_req, nt);
    } else {
        for (int i = nt - 1; i >= 0; i--) {
            if (beta[i] < P.char_scale) break;
            count++;
        }
    }
    return (icm && chains >= 2) ? count : 0;
}

}  // namespace pticm

namespace {

int configure(pticm_ctx* c, bool replay) {
    if (c->configured && c->cfg_replay == replay && c->cfg_nc == c->desc.nc && c->cfg_hist_off == c->desc.hist_off &&
        c->cfg_hist_lo == c->desc.hist_lo && c->cfg_hist_nbins == c->desc.hist_nbins)
        return PTICM_OK;
    std::string msg;
    LaunchConfig cfg;
    if (int rc = choose_config(c->P, c->o, replay, c->desc, cfg, msg)) return fail(rc, msg);
    c->rpc = cfg.rpc;
    c->group = cfg.group;
    c->threads = cfg.threads;
    c->teams = cfg.teams;
    c->block_team = cfg.block_team;
    c->narrow = cfg.narrow;
    c->plan = cfg.plan;
    finish_desc(c->desc, c->P, c->o, cfg);
    if (cfg.state_global || cfg.field_gather) {
        // (with the team scratch in shared memory only the overlap list)
        c->icm_stride = cfg.plan.icm_split ? (long long)(((uint64_t)c->desc.n_pad * 4 + 15) & ~15ull)
                                           : (long long)icm_block_bytes(cfg.teams, c->desc.n_pad);
        const size_t want = (size_t)cfg.group * (size_t)c->icm_stride;
        if (c->d_icm_pool.n != want) CK(c->d_icm_pool.alloc(want));
    }
    std::vector<int32_t> soff, sched;
    single_instance_schedule(cfg.group, soff, sched);
    CK(c->d_sched_off.upload(soff));
    CK(c->d_sched.upload(sched));
    CK(c->d_desc.upload(std::vector<InstanceDesc>{c->desc}));
    c->configured = true;
    c->cfg_replay = replay;
    c->cfg_nc = c->desc.nc;
    c->cfg_hist_off = c->desc.hist_off;
    c->cfg_hist_lo = c->desc.hist_lo;
    c->cfg_hist_nbins = c->desc.hist_nbins;
    return PTICM_OK;
}

EngineArgs make_args(pticm_ctx* c) {
    EngineArgs A{};
    A.desc = c->d_desc.p;
    A.sched_off = c->d_sched_off.p;
    A.sched = c->d_sched.p;
    A.n_inst = 1;
    A.n_blocks = c->group;
    A.row = c->d_row.p;
    A.adj = c->d_adj.p;
    A.col = c->d_col.p;
    A.hpool = c->d_h.p;
    A.beta = c->d_beta.p;
    A.thr = c->d_thr.p;
    A.ptab = c->d_ptab.p;
    A.perm = c->d_perm.p;
    A.spins = c->d_spins.p;
    A.fields = c->d_fields.p;
    A.energy = c->d_E.p;
    A.spins_pub = c->d_pub.p;
    A.spins_pub_half = (long long)c->R * c->desc.n_pad;
    A.energy_pub = c->d_Epub.p;
    A.energy_pub_half = c->R;
    A.flips = c->d_flips.p;
    A.best_E = c->d_bestE.p;
    A.best_sweep = c->d_bestSweep.p;
    A.best_state = c->d_best_state.p;
    A.slot_rep = c->d_slot.p;
    A.xorder = c->d_order.p;
    A.xcursor = c->d_cursor.p;
    A.attempts = c->d_att.p;
    A.successes = c->d_succ.p;
    A.bar = c->d_bar.p;
    A.abort_flag = c->d_abort.p;
    A.status = c->d_status.p;
    A.sweeps = (int)c->o.sweeps;
    A.seed = c->o.seed;
    A.sm = c->plan;
    A.prof = (c->profiling && c->d_prof.n >= (size_t)c->group * PROF_PHASES) ? c->d_prof.p : nullptr;
    A.hist = c->d_hist.p;
    A.obs = c->d_hist.p ? c->d_obs.p : nullptr;
    A.mag_pub = c->d_mag_pub.p;
    A.hist_from = c->hist_from;
    A.flags = engine_flags(c->P, c->o);
    A.icm_pool = c->d_icm_pool.p;
    A.icm_pool_stride = c->icm_stride;
    A.wait_limit_ns = c->wait_limit_ns;
    A.bar_phantom = c->bar_phantom;
    if (c->ebound < 0) c->ebound = energy_bound(c->P);
    A.flag_barrier = c->ebound < (1ll << 31) ? 1 : 0;   // every energy fits the word's 32 bits
    return A;
}

int read_status(pticm_ctx* c, const char* what) {
    DevStatus st{};
    CK(cudaMemcpy(&st, c->d_status.p, sizeof(st), cudaMemcpyDeviceToHost));
    if (st.error) {
        static const char* names[] = {"ok", "group barrier wait expired", "bulk-copy wait expired",
                                      "cluster labelling round cap", "replay trace mismatch", "index out of range",
                                      "aborted"};
        const char* nm = (st.error >= 0 && st.error <= 6) ? names[st.error] : "unknown";
        return fail(PTICM_ERR_DEVICE, std::string(what) + ": device reported " + nm + " at site " +
                                          std::to_string(st.where) + " (" + std::to_string(st.aux0) + ", " +
                                          std::to_string(st.aux1) + ")");
    }
    return PTICM_OK;
}

int reset_flags(pticm_ctx* c) {
    CK(cudaMemsetAsync(c->d_bar.p, 0, c->d_bar.n * sizeof(unsigned), c->stream));
    CK(cudaMemsetAsync(c->d_abort.p, 0, sizeof(int), c->stream));
    CK(cudaMemsetAsync(c->d_status.p, 0, sizeof(DevStatus), c->stream));
    return PTICM_OK;
}

// Fresh bookkeeping after new spins: fields/energies from scratch, best =
// initial state with energy "none yet", identity slot map, shuffled order.
int reset_run_state(pticm_ctx* c) {
    EngineArgs A = make_args(c);
    CK(launch_recompute(A, c->d_rep_inst.p, c->R, 1, nullptr, nullptr, nullptr, c->stream));
    std::vector<long long> be(c->R, kNoBest);
    CK(cudaMemcpyAsync(c->d_bestE.p, be.data(), be.size() * sizeof(long long), cudaMemcpyHostToDevice, c->stream));
    CK(cudaMemcpyAsync(c->d_best_state.p, c->d_spins.p, c->d_spins.n, cudaMemcpyDeviceToDevice, c->stream));
    CK(cudaMemsetAsync(c->d_bestSweep.p, 0, c->R * sizeof(unsigned long long), c->stream));
    CK(cudaMemsetAsync(c->d_flips.p, 0, c->R * sizeof(unsigned long long), c->stream));
    CK(cudaMemsetAsync(c->d_att.p, 0, c->R * sizeof(unsigned long long), c->stream));
    CK(cudaMemsetAsync(c->d_succ.p, 0, c->R * sizeof(unsigned long long), c->stream));
    std::vector<uint32_t> slot(c->R);
    for (int r = 0; r < c->R; r++) slot[r] = (uint32_t)r;
    CK(cudaMemcpyAsync(c->d_slot.p, slot.data(), slot.size() * 4, cudaMemcpyHostToDevice, c->stream));
    std::vector<uint32_t> order(std::max(c->nt, 1), 0);
    for (int k = 0; k + 1 < c->nt; k++) order[k] = (uint32_t)k;
    std::mt19937_64 g(c->o.seed ^ 0x6F72646572ull);
    if (c->nt > 2) std::shuffle(order.begin(), order.begin() + (c->nt - 1), g);
    CK(cudaMemcpyAsync(c->d_order.p, order.data(), order.size() * 4, cudaMemcpyHostToDevice, c->stream));
    CK(cudaStreamSynchronize(c->stream));
    c->steps_done = 0;
    c->attempts = 0;
    c->states_set = true;
    return PTICM_OK;
}

}  // namespace

namespace pticm {
cudaError_t mhist_solve(const MhJob* jobs, int njobs, int max_nt, const uint32_t* hist, const uint64_t* hoff,
                        const uint64_t* hlen, const double* emin, const double* beta, double* logdos, double* logc,
                        float* ldf, double* logZ, unsigned long long* iters, long long max_iters, cudaStream_t st);
}  // namespace pticm

namespace pticm {

// The multihistogram fixed point on the GPU (src/cae_estimator.cc:228-253)
// for any number of histogram sets in one launch (mhist_solve): iterate
// until sum_j ((lnZ_j - lnZ'_j)/lnZ'_j)^2 <= 1e-7, as the reference does.
int mhist_dos_multi(const std::vector<const MhInput*>& in, std::vector<MhOutput>& out) {
    const size_t K = in.size();
    out.assign(K, MhOutput{});
    std::vector<MhJob> jobs;
    std::vector<uint32_t> hist;
    std::vector<uint64_t> hoff, hlen;
    std::vector<double> emin, beta;
    int64_t bins = 0;
    int max_nt = 1;
    std::vector<size_t> solved;
    for (size_t k = 0; k < K; k++) {
        const MhInput& I = *in[k];
        const uint32_t nt = (uint32_t)I.beta.size();
        if (nt < 1 || I.n == 0 || !(I.estep > 0) || I.hoff.size() != nt || I.hlen.size() != nt || I.emin.size() != nt)
            return fail(PTICM_ERR_INVALID, "multihistogram needs samples, rows and estep > 0");
        double me = I.emin[0];
        for (uint32_t j = 1; j < nt; j++) me = std::min(me, I.emin[j]);
        const long long nb = (long long)std::ceil((I.max_emax - me) / I.estep);
        out[k].min_emin = me;
        out[k].logdos.assign((size_t)std::max<long long>(nb, 0), -DBL_MAX);
        out[k].logZ.assign(nt, 0.0);
        out[k].iters = 0;
        if (nb <= 0) continue;
        MhJob J{};
        J.nt = (int32_t)nt;
        J.row0 = (int64_t)beta.size();
        J.nbins = nb;
        J.bin0 = bins;
        J.min_emin = me;
        J.estep = I.estep;
        J.logn = std::log((double)I.n);
        const uint64_t base = hist.size();
        hist.insert(hist.end(), I.hist.begin(), I.hist.end());
        for (uint32_t j = 0; j < nt; j++) {
            hoff.push_back(base + I.hoff[j]);
            hlen.push_back(I.hlen[j]);
        }
        emin.insert(emin.end(), I.emin.begin(), I.emin.end());
        beta.insert(beta.end(), I.beta.begin(), I.beta.end());
        bins += nb;
        max_nt = std::max(max_nt, (int)nt);
        jobs.push_back(J);
        solved.push_back(k);
    }
    if (jobs.empty()) return PTICM_OK;
    DArr<MhJob> d_jobs;
    DArr<uint32_t> d_hist;
    DArr<uint64_t> d_off, d_len;
    DArr<unsigned long long> d_it;
    DArr<double> d_emin, d_beta, d_logZ, d_dos, d_logc;
    DArr<float> d_ldf;
    CK(d_jobs.upload(jobs));
    CK(d_hist.upload(hist, 1));
    CK(d_off.upload(hoff));
    CK(d_len.upload(hlen));
    CK(d_emin.upload(emin));
    CK(d_beta.upload(beta));
    CK(d_logZ.alloc(beta.size()));
    CK(d_dos.alloc((size_t)bins));
    CK(d_logc.alloc((size_t)bins));
    CK(d_ldf.alloc((size_t)bins));
    CK(d_it.alloc(jobs.size()));
    CK(mhist_solve(d_jobs.p, (int)jobs.size(), max_nt, d_hist.p, d_off.p, d_len.p, d_emin.p, d_beta.p, d_dos.p,
                   d_logc.p, d_ldf.p, d_logZ.p, d_it.p, kMhistMaxIters, nullptr));
    CK(cudaDeviceSynchronize());
    std::vector<double> dos, z;
    std::vector<unsigned long long> it;
    CK(d_dos.download(dos));
    CK(d_logZ.download(z));
    CK(d_it.download(it));
    for (size_t q = 0; q < jobs.size(); q++) {
        MhOutput& o = out[solved[q]];
        std::copy(dos.begin() + jobs[q].bin0, dos.begin() + jobs[q].bin0 + jobs[q].nbins, o.logdos.begin());
        std::copy(z.begin() + jobs[q].row0, z.begin() + jobs[q].row0 + jobs[q].nt, o.logZ.begin());
        o.iters = it[q];
        if (o.iters >= (uint64_t)kMhistMaxIters)
            return fail(PTICM_ERR_DEVICE, "multihistogram fixed point did not converge within the iteration cap");
    }
    return PTICM_OK;
}

int mhist_dos_impl(const uint32_t* hist, const uint64_t* hoff, const uint64_t* hlen, uint32_t nt,
                   const double* beta, const double* emin, double estep, uint64_t n, double max_emax,
                   std::vector<double>& logdos, std::vector<double>& logZ, double& min_emin, uint64_t& iters) {
    if (nt < 1 || n == 0 || !(estep > 0)) return fail(PTICM_ERR_INVALID, "multihistogram needs samples, rows and estep > 0");
    MhInput I;
    const uint64_t total = hoff[nt - 1] + hlen[nt - 1];
    I.hist.assign(hist, hist + total);
    I.hoff.assign(hoff, hoff + nt);
    I.hlen.assign(hlen, hlen + nt);
    I.emin.assign(emin, emin + nt);
    I.beta.assign(beta, beta + nt);
    I.estep = estep;
    I.n = n;
    I.max_emax = max_emax;
    std::vector<MhOutput> out;
    if (int rc = mhist_dos_multi({&I}, out)) return rc;
    logdos.swap(out[0].logdos);
    logZ.swap(out[0].logZ);
    min_emin = out[0].min_emin;
    iters = out[0].iters;
    return PTICM_OK;
}

// Per-slot energy histograms of a pilot run -> multihistogram ln g.  Rows of
// slot k (chain c = k / nt, temperature j = k % nt) are merged over chains,
// then cut to [emin_j, emax_j] with bin width estep (make_histogram,
// src/cae_estimator.cc:45-69); n is the sample count of temperature 0,
// accumulated into an int as the reference does.
int compact_slot_hist(const unsigned* rows, int nt, int chains, long long nbins, long long lo, const double* hb,
                      double estep, MhInput& I) {
    I = MhInput{};
    I.hoff.resize(nt);
    I.hlen.resize(nt);
    I.emin.resize(nt);
    I.beta.assign(hb, hb + nt);
    I.estep = estep;
    std::vector<double> emax(nt);
    std::vector<unsigned> merged((size_t)nbins);
    for (int j = 0; j < nt; j++) {
        std::fill(merged.begin(), merged.end(), 0u);
        for (int c = 0; c < chains; c++) {
            const unsigned* row = rows + (size_t)(c * nt + j) * (size_t)nbins;
            for (long long bb = 0; bb < nbins; bb++) merged[bb] += row[bb];
        }
        long long first = -1, last = -1;
        for (long long bb = 0; bb < nbins; bb++)
            if (merged[bb]) { if (first < 0) first = bb; last = bb; }
        if (first < 0) return fail(PTICM_ERR_DEVICE, "pilot run recorded no energies");
        I.emin[j] = (double)(lo + 2 * first);
        emax[j] = (double)(lo + 2 * last);
        I.hlen[j] = (uint64_t)std::ceil((emax[j] - I.emin[j]) / estep) + 1;
        I.hoff[j] = I.hist.size();
        I.hist.resize(I.hist.size() + I.hlen[j], 0);
        for (long long bb = first; bb <= last; bb++)
            if (merged[bb]) I.hist[I.hoff[j] + (uint64_t)std::floor(((double)(lo + 2 * bb) - I.emin[j]) / estep)] += merged[bb];
    }
    int32_t nacc = 0;   // the reference accumulates row 0 into an int
    for (uint64_t k = 0; k < I.hlen[0]; k++) nacc = (int32_t)(nacc + (int32_t)I.hist[I.hoff[0] + k]);
    I.n = (uint64_t)(int64_t)nacc;
    I.max_emax = *std::max_element(emax.begin(), emax.end());
    return PTICM_OK;
}

int slot_hist_dos(const unsigned* rows, int nt, int chains, long long nbins, long long lo, const double* hb,
                  double estep, std::vector<double>& dos, std::vector<double>& logZ, double& min_emin,
                  uint64_t& iters) {
    MhInput I;
    if (int rc = compact_slot_hist(rows, nt, chains, nbins, lo, hb, estep, I)) return rc;
    std::vector<MhOutput> out;
    if (int rc = mhist_dos_multi({&I}, out)) return rc;
    dos.swap(out[0].logdos);
    logZ.swap(out[0].logZ);
    min_emin = out[0].min_emin;
    iters = out[0].iters;
    return PTICM_OK;
}

const HostProblem& problem_host(const pticm_problem* p) { return p->hp; }

int problem_device(const pticm_problem* pc, ProblemDevice* out) {
    pticm_problem* p = const_cast<pticm_problem*>(pc);
    const HostProblem& P = p->hp;
    if (!p->uploaded) {
        CK(p->d_row.upload(P.drow, 4));
        CK(p->d_adj.upload(P.dadj, 4));
        CK(p->d_h.upload(P.dh, 4));
        CK(p->d_perm.upload(P.perm, 4));
        CK(p->d_iperm.upload(P.iperm, 4));
        p->uploaded = true;
    }
    out->row = p->d_row.p;
    out->adj = p->d_adj.p;
    out->h = p->d_h.p;
    out->perm = p->d_perm.p;
    out->iperm = p->d_iperm.p;
    out->n = (int)P.n;
    out->n_pad = pad16(P.n);
    out->kmax = P.kmax;
    out->has_h = P.has_h;
    return PTICM_OK;
}
void set_last_error(const std::string& m) { g_err = m; }

}  // namespace pticm

extern "C" {

const char* pticm_last_error(void) { return g_err.c_str(); }

const char* pticm_version(void) { return "pticm-gb300 0.1 (sm_103a)"; }

int pticm_problem_load_gset(const char* path, pticm_problem** out) {
    if (!path || !out) return fail(PTICM_ERR_INVALID, "null argument");
    auto p = std::make_unique<pticm_problem>();
    std::string msg;
    int rc = parse_gset(path, p->hp, msg);
    if (rc) return fail(rc, msg);
    *out = p.release();
    return PTICM_OK;
}

int pticm_problem_from_coo(int64_t n, int64_t m, const int32_t* src, const int32_t* dst, const double* w,
                           const double* h, pticm_problem** out) {
    if (!out) return fail(PTICM_ERR_INVALID, "null argument");
    auto p = std::make_unique<pticm_problem>();
    std::string msg;
    int rc = problem_from_coo(n, m, src, dst, w, h, p->hp, msg);
    if (rc) return fail(rc, msg);
    *out = p.release();
    return PTICM_OK;
}

int pticm_problem_from_dense(int64_t n, const double* J, const double* h, pticm_problem** out) {
    if (!out) return fail(PTICM_ERR_INVALID, "null argument");
    auto p = std::make_unique<pticm_problem>();
    std::string msg;
    int rc = problem_from_dense(n, J, h, p->hp, msg);
    if (rc) return fail(rc, msg);
    *out = p.release();
    return PTICM_OK;
}

void pticm_problem_free(pticm_problem* p) { delete p; }

int pticm_problem_get_info(const pticm_problem* p, pticm_problem_info* out) {
    if (!p || !out) return fail(PTICM_ERR_INVALID, "null argument");
    const HostProblem& P = p->hp;
    out->n = P.n;
    out->m = P.m;
    out->nnz = (int64_t)P.col.size();
    out->sparse = P.sparse ? 1 : 0;
    out->ncolors = P.ncolors;
    out->kmax = P.kmax;
    out->has_linear = P.has_h ? 1 : 0;
    out->char_scale = P.char_scale;
    out->total_weight = P.total_weight;
    return PTICM_OK;
}

int pticm_problem_get_colouring(const pticm_problem* p, int32_t* colour) {
    if (!p || !colour) return fail(PTICM_ERR_INVALID, "null argument");
    const HostProblem& P = p->hp;
    for (int32_t c = 0; c < P.ncolors; c++)
        for (int32_t d = P.color_off[c]; d < P.color_off[c + 1]; d++) colour[P.perm[d]] = c;
    return PTICM_OK;
}

int pticm_problem_evaluate(const pticm_problem* pc, int64_t count, const uint8_t* states, double* energy,
                           double* maxcut, double* dE) {
    if (!pc || count < 0 || (count > 0 && !states)) return fail(PTICM_ERR_INVALID, "invalid arguments");
    if (int rc = check_device()) return rc;
    if (count == 0) return PTICM_OK;
    pticm_problem* p = const_cast<pticm_problem*>(pc);
    const HostProblem& P = p->hp;
    const int n = (int)P.n, npad = pad16(n);
    ProblemDevice PD;
    if (int rc = problem_device(p, &PD)) return rc;
    std::vector<int8_t> dev((size_t)count * npad, 1);
    for (int64_t g = 0; g < count; g++)
        for (int i = 0; i < n; i++) dev[g * npad + i] = states[g * n + P.perm[i]] ? 1 : -1;
    DArr<int8_t> d_s;
    DArr<long long> d_E, d_c;
    DArr<int32_t> d_dE;
    CK(d_s.upload(dev));
    CK(d_E.alloc(count));
    CK(d_c.alloc(count));
    if (dE) CK(d_dE.alloc((size_t)count * npad));
    CK(launch_evaluate(p->d_row.p, p->d_adj.p, P.has_h ? p->d_h.p : nullptr, n, npad, d_s.p, (int)count, d_E.p,
                       d_c.p, dE ? d_dE.p : nullptr, nullptr));
    CK(cudaDeviceSynchronize());
    std::vector<long long> E, C2;
    CK(d_E.download(E));
    CK(d_c.download(C2));
    for (int64_t g = 0; g < count; g++) {
        if (energy) energy[g] = (double)E[g];
        if (maxcut) maxcut[g] = 0.5 * (double)C2[g];
    }
    if (dE) {
        std::vector<int32_t> d;
        CK(d_dE.download(d));
        for (int64_t g = 0; g < count; g++)
            for (int i = 0; i < n; i++) dE[g * n + P.perm[i]] = (double)d[g * npad + i];
    }
    return PTICM_OK;
}

void pticm_opts_default(pticm_opts* o) {
    if (!o) return;
    std::memset(o, 0, sizeof(*o));
    o->seed = 0;
    o->nt = 20;
    o->chains = 2;
    o->sweeps = 1;
    o->icm = 0;
    o->exchange = 1;
    o->best_per_phase = 0;
    o->icm_algo = 0;
}

int pticm_beta_linspace(double* beta, double T0, double T1, uint64_t nt, int inverse) {
    if (!beta || nt < 2) return fail(PTICM_ERR_INVALID, "need at least two temperatures");
    beta_linspace(beta, T0, T1, nt, inverse != 0);
    return PTICM_OK;
}

int pticm_create(const pticm_problem* p, const pticm_opts* o, pticm_ctx** out) {
    if (!p || !o || !out) return fail(PTICM_ERR_INVALID, "null argument");
    if (o->nt < 2) return fail(PTICM_ERR_INVALID, "at least two temperatures are needed");
    if (o->chains < 1 || o->chains > 16) return fail(PTICM_ERR_INVALID, "chains must be in [1, 16]");
    if (o->icm && (o->chains % 2)) return fail(PTICM_ERR_INVALID, "ICM pairs chains: use an even chain count");
    if (o->sweeps < 1) return fail(PTICM_ERR_INVALID, "sweeps must be >= 1");
    if (o->exchange > 1) return fail(PTICM_ERR_INVALID, "exchange must be 0 or 1");
    if (o->icm_algo > 3) return fail(PTICM_ERR_INVALID, "icm_algo must be in 0..3");
    if (int rc = check_device()) return rc;
    auto c = std::make_unique<pticm_ctx>();
    c->P = p->hp;
    c->o = *o;
    c->nt = (int)o->nt;
    c->C = (int)o->chains;
    c->R = c->nt * c->C;
    const HostProblem& P = c->P;
    InstanceDesc& D = c->desc;
    D.n = (int32_t)P.n;
    D.n_pad = pad16(P.n);
    D.nnz = (int32_t)P.dadj.size();
    D.ncolors = P.ncolors;
    D.kmax = P.kmax;
    D.nt = c->nt;
    D.chains = c->C;
    D.R = c->R;
    D.nc = 0;
    D.has_h = P.has_h ? 1 : 0;
    CK(cudaStreamCreateWithFlags(&c->stream, cudaStreamNonBlocking));
    CK(cudaEventCreate(&c->ev0));
    CK(cudaEventCreate(&c->ev1));
    CK(c->d_row.upload(P.drow, 4));
    CK(c->d_adj.upload(P.dadj, 4));
    CK(c->d_col.upload(P.color_off, 4));
    CK(c->d_h.upload(P.dh, 4));
    CK(c->d_perm.upload(P.iperm, 4));   // original site -> device site
    const size_t spins = (size_t)c->R * D.n_pad;
    CK(c->d_spins.alloc(spins));
    CK(c->d_fields.alloc(spins));
    CK(c->d_best_state.alloc(spins));
    CK(c->d_pub.alloc(2 * spins));
    CK(c->d_E.alloc(c->R));
    CK(c->d_Epub.alloc(2 * c->R * kPubStride));
    CK(c->d_bestE.alloc(c->R));
    CK(c->d_flips.alloc(c->R));
    CK(c->d_bestSweep.alloc(c->R));
    CK(c->d_att.alloc(c->R));
    CK(c->d_succ.alloc(c->R));
    CK(c->d_slot.alloc(c->R));
    CK(c->d_order.alloc(std::max(c->nt, 1)));
    CK(c->d_cursor.alloc(1));
    CK(c->d_bar.alloc(2));
    CK(c->d_abort.alloc(1));
    CK(c->d_status.alloc(1));
    CK(c->d_mismatch.alloc(1));
    std::vector<int32_t> ri(c->R, 0);
    CK(c->d_rep_inst.upload(ri));
    CK(c->d_desc.upload(std::vector<InstanceDesc>{D}));
    *out = c.release();
    return PTICM_OK;
}

void pticm_destroy(pticm_ctx* c) { delete c; }

int pticm_set_ladder(pticm_ctx* c, const double* beta, uint32_t nt, int32_t nc) {
    if (!c || !beta) return fail(PTICM_ERR_INVALID, "null argument");
    if ((int)nt != c->nt) return fail(PTICM_ERR_INVALID, "ladder length differs from the context's nt");
    for (uint32_t k = 0; k < nt; k++)
        if (!std::isfinite(beta[k])) return fail(PTICM_ERR_INVALID, "non-finite inverse temperature");
    c->beta.assign(beta, beta + nt);
    std::vector<uint32_t> thr;
    std::vector<double> ptab;
    c->nc = ladder_tables(c->P, beta, c->nt, nc, c->o.icm != 0, c->C, thr, ptab);
    c->desc.nc = c->nc;
    CK(c->d_beta.upload(c->beta));
    CK(c->d_thr.upload(thr, 4));
    CK(c->d_ptab.upload(ptab, 4));
    c->ladder_set = true;
    return PTICM_OK;
}

int pticm_set_states(pticm_ctx* c, const uint8_t* states) {
    if (!c || !states) return fail(PTICM_ERR_INVALID, "null argument");
    const HostProblem& P = c->P;
    const int n = (int)P.n, npad = c->desc.n_pad;
    // the caller's bytes go to the device as they are; a kernel moves them
    // into the device site order
    const size_t bytes = (size_t)c->R * (size_t)n;
    if (c->d_states_in.n != bytes) CK(c->d_states_in.alloc(bytes));
    CK(cudaMemcpyAsync(c->d_states_in.p, states, bytes, cudaMemcpyHostToDevice, c->stream));
    CK(launch_load_states(c->d_states_in.p, c->d_perm.p, c->d_spins.p, c->R, n, npad, c->stream));
    if (int rc = configure(c, false)) return rc;
    return reset_run_state(c);
}

int pticm_init_states(pticm_ctx* c, uint64_t seed) {
    if (!c) return fail(PTICM_ERR_INVALID, "null argument");
    if (int rc = configure(c, false)) return rc;
    EngineArgs A = make_args(c);
    CK(launch_init_spins(A, c->d_rep_inst.p, c->R, seed, c->stream));
    return reset_run_state(c);
}

int pticm_run(pticm_ctx* c, uint64_t pt_steps, uint32_t phase_mask) {
    if (!c) return fail(PTICM_ERR_INVALID, "null argument");
    if (!c->ladder_set) return fail(PTICM_ERR_INVALID, "set a ladder before running");
    if (!c->states_set) return fail(PTICM_ERR_INVALID, "initialise the replica states before running");
    if (phase_mask == 0 || phase_mask > 7) return fail(PTICM_ERR_INVALID, "phase_mask must be in 1..7");
    if (int rc = configure(c, false)) return rc;
    c->last_ms = 0.0;
    uint64_t left = pt_steps;
    while (left > 0) {
        const int chunk = (int)std::min<uint64_t>(left, 1u << 16);
        if (int rc = reset_flags(c)) return rc;
        EngineArgs A = make_args(c);
        A.step0 = c->steps_done;
        A.nsteps = chunk;
        A.phase_mask = (int)phase_mask;
        CK(cudaEventRecord(c->ev0, c->stream));
        CK(launch_engine(A, c->threads, false, c->block_team, c->narrow, c->group > 1, c->stream));
        CK(cudaEventRecord(c->ev1, c->stream));
        CK(cudaEventSynchronize(c->ev1));
        float ms = 0.f;
        CK(cudaEventElapsedTime(&ms, c->ev0, c->ev1));
        c->last_ms += ms;
        if (int rc = read_status(c, "pticm_run")) return rc;
        c->steps_done += (uint64_t)chunk;
        if (phase_mask & PHASE_SWEEP) c->attempts += (uint64_t)chunk * c->o.sweeps * (uint64_t)c->R * (uint64_t)c->P.n;
        left -= (uint64_t)chunk;
    }
    return PTICM_OK;
}

int pticm_icm_pairs(pticm_ctx* c, const int64_t* seeds, uint32_t count, int exact) {
    if (!c || !seeds) return fail(PTICM_ERR_INVALID, "null argument");
    if (!c->ladder_set || !c->states_set) return fail(PTICM_ERR_INVALID, "set the ladder and the states first");
    const uint32_t pairs = (uint32_t)(c->nc * (c->C / 2));
    if (count != pairs)
        return fail(PTICM_ERR_INVALID, "expected one seed per ICM pair (" + std::to_string(pairs) + ")");
    if (pairs == 0) return PTICM_OK;
    for (uint32_t q = 0; q < count; q++)
        if (seeds[q] < -2 || seeds[q] >= c->P.n)
            return fail(PTICM_ERR_INVALID, "seed " + std::to_string(seeds[q]) + " of pair " + std::to_string(q) +
                                               " is neither a site, -1 (random) nor -2 (skip)");
    if (int rc = configure(c, false)) return rc;
    std::vector<long long> f(seeds, seeds + count);
    CK(c->d_icm_force.upload(f));
    if (int rc = reset_flags(c)) return rc;
    EngineArgs A = make_args(c);
    A.step0 = c->steps_done;
    A.nsteps = 1;
    A.phase_mask = PHASE_ICM;
    A.icm_force = c->d_icm_force.p;
    A.icm_exact = exact ? 1 : 0;
    CK(launch_engine(A, c->threads, false, c->block_team, c->narrow, c->group > 1, c->stream));
    CK(cudaStreamSynchronize(c->stream));
    DevStatus st{};
    CK(cudaMemcpy(&st, c->d_status.p, sizeof(st), cudaMemcpyDeviceToHost));
    if (st.error == DEV_BAD_INDEX && st.where == 36)   // ICM site 30 + 6: a seed outside the overlap
        return fail(PTICM_ERR_INVALID, "the seed of pair " + std::to_string(st.aux0) +
                                           " is not a site where the pair's states differ");
    if (int rc = read_status(c, "pticm_icm_pairs")) return rc;
    c->steps_done += 1;
    return PTICM_OK;
}

int pticm_get_layout(pticm_ctx* c, pticm_layout* out) {
    if (!c || !out) return fail(PTICM_ERR_INVALID, "null argument");
    if (!c->configured) return fail(PTICM_ERR_INVALID, "the layout is chosen with the first states");
    out->replicas_per_block = (uint32_t)c->rpc;
    out->blocks = (uint32_t)c->group;
    out->threads = (uint32_t)c->threads;
    out->icm_teams = (uint32_t)c->teams;
    out->block_team = c->block_team ? 1 : 0;
    out->narrow = c->narrow ? 1 : 0;
    out->adjacency_staged = c->plan.stage_adj;
    out->state_mode = c->plan.state_global ? 2 : (c->plan.field_gather ? 1 : 0);
    return PTICM_OK;
}

int pticm_get_exchange_order(pticm_ctx* c, uint32_t* order) {
    if (!c || !order) return fail(PTICM_ERR_INVALID, "null argument");
    CK(cudaStreamSynchronize(c->stream));
    std::vector<uint32_t> o;
    CK(c->d_order.download(o));
    for (int k = 0; k + 1 < c->nt; k++) order[k] = o[k];
    return PTICM_OK;
}

int pticm_set_wait_limit(pticm_ctx* c, uint64_t limit_ns, uint32_t phantom_arrivals) {
    if (!c) return fail(PTICM_ERR_INVALID, "null argument");
    if (limit_ns > 60ull * 1000000000ull) return fail(PTICM_ERR_INVALID, "wait limit above 60 s");
    if (phantom_arrivals > 1) return fail(PTICM_ERR_INVALID, "phantom_arrivals must be 0 or 1");
    c->wait_limit_ns = limit_ns;
    c->bar_phantom = (int)phantom_arrivals;
    return PTICM_OK;
}

int pticm_replay(pticm_ctx* c, const pticm_trace* t) {
    if (!c || !t) return fail(PTICM_ERR_INVALID, "null argument");
    if (c->C != 2) return fail(PTICM_ERR_INVALID, "replay follows the reference: two chains");
    if (!c->ladder_set || !c->states_set) return fail(PTICM_ERR_INVALID, "set the ladder and the states first");
    for (int k = 0; k + 1 < c->nt; k++)
        for (int j = k + 1; j < c->nt; j++)
            if (std::fabs(c->beta[k] - c->beta[j]) < 1e-10)
                return fail(PTICM_ERR_UNSUPPORTED, "replay needs distinct temperatures");
    if (int rc = configure(c, true)) return rc;
    const uint64_t steps = t->pt_steps;
    const uint64_t nsw = steps * c->o.sweeps * (uint64_t)c->R;
    DArr<double> d_u, d_logu;
    DArr<uint64_t> d_off;
    DArr<int32_t> d_xs;
    DArr<int64_t> d_seed;
    std::vector<double> u(t->uniforms, t->uniforms + t->n_uniforms);
    std::vector<uint64_t> off(t->sweep_offsets, t->sweep_offsets + nsw + 1);
    const uint64_t nx = steps * 2 * (uint64_t)(c->nt - 1);
    std::vector<int32_t> xs(t->xchg_slot, t->xchg_slot + nx);
    std::vector<double> xl(t->xchg_logu, t->xchg_logu + nx);
    const uint64_t ni = steps * (uint64_t)c->nc;
    std::vector<int64_t> seeds;
    if (ni) seeds.assign(t->icm_seed, t->icm_seed + ni);
    CK(d_u.upload(u, 1));
    CK(d_off.upload(off));
    CK(d_xs.upload(xs, 1));
    CK(d_logu.upload(xl, 1));
    CK(d_seed.upload(seeds, 1));
    if (int rc = reset_flags(c)) return rc;
    EngineArgs A = make_args(c);
    A.step0 = c->steps_done;
    A.nsteps = (int)steps;
    A.phase_mask = PHASE_SWEEP | PHASE_EXCHANGE | (c->nc ? PHASE_ICM : 0);
    A.flags = ENGINE_REPLAY | (A.flags & ENGINE_ICM_MASK);
    A.replay.uniforms = d_u.p;
    A.replay.sweep_offsets = reinterpret_cast<const uint64_t*>(d_off.p);
    A.replay.xchg_slot = d_xs.p;
    A.replay.xchg_logu = d_logu.p;
    A.replay.icm_seed = reinterpret_cast<const int64_t*>(d_seed.p);
    A.replay.n_uniforms = u.size();
    A.replay.n_xchg = xs.size();
    A.replay.n_icm = seeds.size();
    CK(cudaEventRecord(c->ev0, c->stream));
    CK(launch_engine(A, c->threads, true, false, false, false, c->stream));
    CK(cudaEventRecord(c->ev1, c->stream));
    CK(cudaEventSynchronize(c->ev1));
    float ms = 0.f;
    CK(cudaEventElapsedTime(&ms, c->ev0, c->ev1));
    c->last_ms = ms;
    if (int rc = read_status(c, "pticm_replay")) return rc;
    c->steps_done += steps;
    c->attempts += steps * c->o.sweeps * (uint64_t)c->R * (uint64_t)c->P.n;
    return PTICM_OK;
}

int pticm_get_stats(pticm_ctx* c, pticm_stats* s, uint64_t* swap_attempts, uint64_t* swap_successes) {
    if (!c) return fail(PTICM_ERR_INVALID, "null argument");
    CK(cudaStreamSynchronize(c->stream));
    std::vector<unsigned long long> fl, at, su;
    CK(c->d_flips.download(fl));
    CK(c->d_att.download(at));
    CK(c->d_succ.download(su));
    if (s) {
        s->pt_steps = c->steps_done;
        s->attempts = c->attempts;
        s->flips = 0;
        for (auto v : fl) s->flips += v;
        s->swaps = 0;
        for (auto v : su) s->swaps += v;
        s->nt = (uint32_t)c->nt;
        s->chains = (uint32_t)c->C;
        s->nc = (uint32_t)c->nc;
        s->replicas = (uint32_t)c->R;
        s->last_run_ms = c->last_ms;
    }
    for (int k = 0; k < c->R; k++) {
        if (swap_attempts) swap_attempts[k] = at[k];
        if (swap_successes) swap_successes[k] = su[k];
    }
    return PTICM_OK;
}

int pticm_get_best(pticm_ctx* c, double* energy, uint64_t* sweep, uint8_t* state, int64_t* replica) {
    if (!c) return fail(PTICM_ERR_INVALID, "null argument");
    CK(cudaStreamSynchronize(c->stream));
    std::vector<long long> be;
    std::vector<unsigned long long> bs;
    CK(c->d_bestE.download(be));
    CK(c->d_bestSweep.download(bs));
    int64_t bi = -1;
    long long best = kNoBest;
    for (int r = 0; r < c->R; r++)
        if (be[r] < best) { best = be[r]; bi = r; }
    if (energy) *energy = (bi < 0) ? DBL_MAX : (double)best;
    if (sweep) *sweep = (bi < 0) ? 0 : bs[bi];
    if (replica) *replica = bi;
    if (state) {
        const int n = (int)c->P.n, npad = c->desc.n_pad;
        std::vector<int8_t> row(npad, 1);
        if (bi >= 0) CK(cudaMemcpy(row.data(), c->d_best_state.p + (size_t)bi * npad, npad, cudaMemcpyDeviceToHost));
        for (int i = 0; i < n; i++) state[c->P.perm[i]] = row[i] > 0 ? 1 : 0;
    }
    return PTICM_OK;
}

int pticm_get_replicas(pticm_ctx* c, uint8_t* states, int64_t* energy, int32_t* fields, uint32_t* slot_of_replica) {
    if (!c) return fail(PTICM_ERR_INVALID, "null argument");
    CK(cudaStreamSynchronize(c->stream));
    const int n = (int)c->P.n, npad = c->desc.n_pad;
    if (states) {
        std::vector<int8_t> s;
        CK(c->d_spins.download(s));
        for (int r = 0; r < c->R; r++)
            for (int i = 0; i < n; i++) states[(size_t)r * n + c->P.perm[i]] = s[(size_t)r * npad + i] > 0 ? 1 : 0;
    }
    if (fields) {
        std::vector<int32_t> f;
        CK(c->d_fields.download(f));
        for (int r = 0; r < c->R; r++)
            for (int i = 0; i < n; i++) fields[(size_t)r * n + c->P.perm[i]] = f[(size_t)r * npad + i];
    }
    if (energy) {
        std::vector<long long> e;
        CK(c->d_E.download(e));
        for (int r = 0; r < c->R; r++) energy[r] = e[r];
    }
    if (slot_of_replica) {
        std::vector<uint32_t> sl;
        CK(c->d_slot.download(sl));
        for (int s = 0; s < c->R; s++) slot_of_replica[sl[s]] = (uint32_t)s;
    }
    return PTICM_OK;
}

int pticm_get_ladder(pticm_ctx* c, double* beta, uint32_t* slot_to_replica, uint32_t* nc) {
    if (!c) return fail(PTICM_ERR_INVALID, "null argument");
    if (beta) for (int k = 0; k < c->nt; k++) beta[k] = c->beta.empty() ? 0.0 : c->beta[k];
    if (nc) *nc = (uint32_t)c->nc;
    if (slot_to_replica) {
        CK(cudaStreamSynchronize(c->stream));
        std::vector<uint32_t> sl;
        CK(c->d_slot.download(sl));
        for (int s = 0; s < c->R; s++) slot_to_replica[s] = sl[s];
    }
    return PTICM_OK;
}

int pticm_verify(pticm_ctx* c, uint64_t* mismatches) {
    if (!c || !mismatches) return fail(PTICM_ERR_INVALID, "null argument");
    if (!c->states_set) return fail(PTICM_ERR_INVALID, "no states yet");
    CK(cudaMemsetAsync(c->d_mismatch.p, 0, sizeof(unsigned long long), c->stream));
    EngineArgs A = make_args(c);
    CK(launch_recompute(A, c->d_rep_inst.p, c->R, 0, c->d_mismatch.p, nullptr, nullptr, c->stream));
    unsigned long long mm = 0;
    CK(cudaMemcpyAsync(&mm, c->d_mismatch.p, sizeof(mm), cudaMemcpyDeviceToHost, c->stream));
    CK(cudaStreamSynchronize(c->stream));
    *mismatches = mm;
    return PTICM_OK;
}

int pticm_set_profiling(pticm_ctx* c, int enable) {
    if (!c) return fail(PTICM_ERR_INVALID, "null argument");
    c->profiling = enable != 0;
    if (c->profiling) CK(c->d_prof.alloc((size_t)std::max(c->R, 1) * PROF_PHASES));
    return PTICM_OK;
}

int pticm_get_profile(pticm_ctx* c, double* mean_ms, double* max_ms) {
    static_assert(PROF_PHASES == PTICM_PROFILE_SLOTS, "profile slots");
    if (!c) return fail(PTICM_ERR_INVALID, "null argument");
    if (!c->profiling) return fail(PTICM_ERR_INVALID, "profiling is not enabled");
    CK(cudaStreamSynchronize(c->stream));
    std::vector<unsigned long long> v;
    CK(c->d_prof.download(v));
    int dev = 0, khz = 0;
    CK(cudaGetDevice(&dev));
    CK(cudaDeviceGetAttribute(&khz, cudaDevAttrClockRate, dev));
    const double to_ms = 1.0 / (double)std::max(khz, 1);
    const int blocks = std::max(c->group, 1);
    for (int q = 0; q < PROF_PHASES; q++) {
        double sum = 0, mx = 0;
        for (int b = 0; b < blocks; b++) {
            const double raw = (double)v[(size_t)b * PROF_PHASES + q];
            const double x = q == PROF_ICM_COUNT ? raw : raw * to_ms;
            sum += x;
            mx = std::max(mx, x);
        }
        if (mean_ms) mean_ms[q] = sum / blocks;
        if (max_ms) max_ms[q] = mx;
    }
    return PTICM_OK;
}

int pticm_enable_energy_histograms(pticm_ctx* c, uint64_t from_step) {
    if (!c) return fail(PTICM_ERR_INVALID, "null argument");
    // every energy lies in [-W, W], W = sum |J| over edges + sum |h|, and has
    // the parity of W: bins of width 2 from -W are exact energy levels
    const long long wabs = energy_bound(c->P);
    if ((unsigned long long)(wabs + 1) * (unsigned long long)c->R > (1ull << 31))
        return fail(PTICM_ERR_UNSUPPORTED, "energy range too large for per-slot histograms");
    c->hist_lo = -wabs;
    c->hist_nbins = wabs + 1;
    c->hist_from = from_step;
    c->desc.hist_off = 0;
    c->desc.hist_lo = c->hist_lo;
    c->desc.hist_nbins = c->hist_nbins;
    CK(c->d_hist.alloc((size_t)c->R * (size_t)c->hist_nbins));
    CK(c->d_obs.alloc(2 * (size_t)c->R));
    CK(c->d_mag_pub.alloc(2 * (size_t)c->R));
    return PTICM_OK;
}

int pticm_get_observables(pticm_ctx* c, double* T, double* C, double* X, double* u, double* m, uint64_t* samples) {
    if (!c) return fail(PTICM_ERR_INVALID, "null argument");
    if (!c->d_hist.p) return fail(PTICM_ERR_INVALID, "energy histograms are not enabled");
    CK(cudaStreamSynchronize(c->stream));
    std::vector<unsigned> h;
    std::vector<long long> o;
    CK(c->d_hist.download(h));
    CK(c->d_obs.download(o));
    const double n = (double)c->P.n;
    for (int j = 0; j < c->nt; j++) {
        double cnt = 0, se = 0, se2 = 0, sm = 0, sm2 = 0;
        for (int ch = 0; ch < c->C; ch++) {
            const int k = ch * c->nt + j;
            const unsigned* row = h.data() + (size_t)k * (size_t)c->hist_nbins;
            for (long long b = 0; b < c->hist_nbins; b++) {
                if (!row[b]) continue;
                const double E = (double)(c->hist_lo + 2 * b);
                cnt += row[b];
                se += row[b] * E;
                se2 += row[b] * E * E;
            }
            sm += (double)o[2 * k];
            sm2 += (double)o[2 * k + 1];
        }
        const double beta = c->beta.empty() ? 0.0 : c->beta[j];
        const double eA = cnt > 0 ? se / cnt : 0.0, e2 = cnt > 0 ? se2 / cnt : 0.0;
        const double mA = cnt > 0 ? sm / cnt : 0.0, m2 = cnt > 0 ? sm2 / cnt : 0.0;
        if (T) T[j] = beta != 0.0 ? 1.0 / beta : 0.0;
        if (C) C[j] = beta * beta * (e2 - eA * eA) / n;
        if (X) X[j] = beta * (m2 - mA * mA) / n;
        if (u) u[j] = eA / n;
        if (m) m[j] = mA / n;
        if (samples) samples[j] = (uint64_t)cnt;
    }
    return PTICM_OK;
}

int pticm_get_energy_histograms(pticm_ctx* c, uint32_t* hist, int64_t* e_lo, uint64_t* nbins) {
    if (!c) return fail(PTICM_ERR_INVALID, "null argument");
    if (!c->d_hist.p) return fail(PTICM_ERR_INVALID, "energy histograms are not enabled");
    if (e_lo) *e_lo = c->hist_lo;
    if (nbins) *nbins = (uint64_t)c->hist_nbins;
    if (hist) {
        CK(cudaStreamSynchronize(c->stream));
        CK(cudaMemcpy(hist, c->d_hist.p, c->d_hist.n * sizeof(unsigned), cudaMemcpyDeviceToHost));
    }
    return PTICM_OK;
}

int pticm_mhist_dos(const uint32_t* hist, const uint64_t* hist_off, const uint64_t* hist_len, uint32_t nt,
                    const double* beta_hist, const double* emin, double estep, uint64_t n, double max_emax,
                    double* logdos, uint64_t logdos_cap, double* logZ, uint64_t* nbins, uint64_t* iterations) {
    if (!hist || !hist_off || !hist_len || !beta_hist || !emin || !nbins) return fail(PTICM_ERR_INVALID, "null argument");
    if (int rc = check_device()) return rc;
    std::vector<double> dos, z;
    double min_emin = 0;
    uint64_t it = 0;
    if (int rc = mhist_dos_impl(hist, hist_off, hist_len, nt, beta_hist, emin, estep, n, max_emax, dos, z, min_emin, it))
        return rc;
    *nbins = dos.size();
    if (logdos) std::copy(dos.begin(), dos.begin() + std::min<uint64_t>(logdos_cap, dos.size()), logdos);
    if (logZ) std::copy(z.begin(), z.end(), logZ);
    if (iterations) *iterations = it;
    return PTICM_OK;
}

int pticm_cae_walk(const double* logdos, uint64_t nbins, double min_emin, double estep, double beta_start,
                   double beta_end, double step_size, double r, uint32_t num_temps, double* beta_out, uint32_t* count) {
    if (!logdos || !beta_out || !count || num_temps < 1) return fail(PTICM_ERR_INVALID, "invalid arguments");
    std::vector<double> dos(logdos, logdos + nbins);
    *count = cae_walk(dos, min_emin, estep, beta_start, beta_end, step_size, r, num_temps, beta_out);
    return PTICM_OK;
}

int pticm_cae_ladder(const pticm_problem* p, uint64_t seed, double T0, double T1, int inverse, uint32_t nt,
                     double estep, double step_size, double r, uint64_t samples, uint64_t burn_in,
                     double* beta_out, uint32_t* count) {
    if (!p || !beta_out || !count || nt < 2 || samples == 0 || !(estep > 0))
        return fail(PTICM_ERR_INVALID, "invalid arguments");
    if (int rc = check_device()) return rc;
    // histogram temperatures: linear in beta from the largest beta down
    // (src/cae_estimator.cc:308-328)
    double beta_start = inverse ? T0 : 1 / T0, beta_end = inverse ? T1 : 1 / T1;
    if (beta_start < beta_end) std::swap(beta_start, beta_end);
    const double beta_step = (beta_end - beta_start) / (double)(nt - 1);
    std::vector<double> hb(nt);
    double b = beta_start;
    for (uint32_t i = 0; i < nt; i++, b += beta_step) hb[i] = b;
    // pilot run (gather_samples, :76-151): one chain, no ICM, shuffled-order exchange
    pticm_opts o;
    pticm_opts_default(&o);
    o.seed = seed;
    o.nt = nt;
    o.chains = 1;
    o.icm = 0;
    o.exchange = 0;
    pticm_ctx* c = nullptr;
    if (int rc = pticm_create(p, &o, &c)) return rc;
    std::unique_ptr<pticm_ctx> hold(c);
    if (int rc = pticm_set_ladder(c, hb.data(), nt, 0)) return rc;
    if (int rc = pticm_init_states(c, seed)) return rc;
    if (int rc = pticm_enable_energy_histograms(c, burn_in)) return rc;
    if (int rc = pticm_run(c, burn_in + samples, 7)) return rc;
    std::vector<unsigned> habs;
    CK(c->d_hist.download(habs));
    std::vector<double> dos, z;
    double min_emin = 0;
    uint64_t it = 0;
    if (int rc = slot_hist_dos(habs.data(), (int)nt, 1, c->hist_nbins, c->hist_lo, hb.data(), estep, dos, z,
                               min_emin, it))
        return rc;
    *count = cae_walk(dos, min_emin, estep, beta_start, beta_end, step_size, r, nt, beta_out);
    return PTICM_OK;
}

// ------------------------------------------------------------ checkpoints
// File: "PTICMCKP", u32 version, u32 0; u64 header words (problem and option
// identity, counters); nc; the ladder; the histogram range; then each device
// array as u64 byte count + bytes, in a fixed order.
}  // extern "C"

namespace {

constexpr uint32_t kCkptVersion = 1;

struct CkptFile {
    FILE* f = nullptr;
    bool ok = true;
    ~CkptFile() {
        if (f) fclose(f);
    }
    void put(const void* p, size_t n) { ok = ok && fwrite(p, 1, n, f) == n; }
    void get(void* p, size_t n) { ok = ok && fread(p, 1, n, f) == n; }
    template <class T>
    void put_val(T v) { put(&v, sizeof v); }
    template <class T>
    T get_val() {
        T v{};
        get(&v, sizeof v);
        return v;
    }
};

// FNV-1a over the problem's size, adjacency, couplings and linear terms.
uint64_t problem_fingerprint(const HostProblem& P) {
    uint64_t h = 1469598103934665603ull;
    auto mix = [&](const void* p, size_t n) {
        const unsigned char* b = static_cast<const unsigned char*>(p);
        for (size_t i = 0; i < n; i++) h = (h ^ b[i]) * 1099511628211ull;
    };
    mix(&P.n, sizeof P.n);
    mix(P.row.data(), P.row.size() * sizeof(int64_t));
    mix(P.col.data(), P.col.size() * sizeof(int32_t));
    mix(P.w.data(), P.w.size() * sizeof(int32_t));
    mix(P.h.data(), P.h.size() * sizeof(int32_t));
    return h;
}

// the identity a checkpoint must share with the context it is loaded into
std::vector<uint64_t> ckpt_identity(const pticm_ctx* c) {
    return {(uint64_t)c->P.n, (uint64_t)c->P.col.size(), (uint64_t)c->R,       (uint64_t)c->nt,
            (uint64_t)c->C,   c->o.seed,                  (uint64_t)c->o.sweeps, (uint64_t)c->o.icm,
            (uint64_t)c->o.exchange, (uint64_t)c->o.best_per_phase, problem_fingerprint(c->P)};
}

template <class T>
int ckpt_dump(CkptFile& F, const DArr<T>& a) {
    std::vector<T> v;
    CK(a.download(v));
    F.put_val<uint64_t>(v.size() * sizeof(T));
    F.put(v.data(), v.size() * sizeof(T));
    return PTICM_OK;
}

template <class T>
int ckpt_read(CkptFile& F, const DArr<T>& a, const char* what, std::vector<T>& v) {
    const uint64_t bytes = F.get_val<uint64_t>();
    if (!F.ok || bytes != a.n * sizeof(T))
        return fail(PTICM_ERR_INVALID, std::string("checkpoint: ") + what + " does not match the context");
    v.assign(a.n, T{});
    F.get(v.data(), bytes);
    if (!F.ok) return fail(PTICM_ERR_IO, std::string("checkpoint: short read in ") + what);
    return PTICM_OK;
}

template <class T>
int ckpt_restore(CkptFile& F, DArr<T>& a, const char* what) {
    std::vector<T> v;
    if (int rc = ckpt_read(F, a, what, v)) return rc;
    if (!v.empty()) CK(cudaMemcpy(a.p, v.data(), v.size() * sizeof(T), cudaMemcpyHostToDevice));
    return PTICM_OK;
}

// The engine indexes with the slot map and the exchange order: a map read
// from a file must be a permutation (of 0..count-1) before it is uploaded.
bool is_permutation_of_range(const uint32_t* v, size_t count) {
    std::vector<char> seen(count, 0);
    for (size_t i = 0; i < count; i++) {
        if (v[i] >= count || seen[v[i]]) return false;
        seen[v[i]] = 1;
    }
    return true;
}

int ckpt_restore_permutation(CkptFile& F, DArr<uint32_t>& a, size_t count, const char* what) {
    std::vector<uint32_t> v;
    if (int rc = ckpt_read(F, a, what, v)) return rc;
    if (count > v.size() || !is_permutation_of_range(v.data(), count))
        return fail(PTICM_ERR_INVALID, std::string("checkpoint: ") + what + " is not a permutation");
    if (!v.empty()) CK(cudaMemcpy(a.p, v.data(), v.size() * sizeof(uint32_t), cudaMemcpyHostToDevice));
    return PTICM_OK;
}

}  // namespace

extern "C" {

int pticm_checkpoint_save(pticm_ctx* c, const char* path) {
    if (!c || !path) return fail(PTICM_ERR_INVALID, "null argument");
    if (!c->ladder_set || !c->states_set) return fail(PTICM_ERR_INVALID, "nothing to save: set a ladder and states");
    CK(cudaStreamSynchronize(c->stream));
    CkptFile F;
    F.f = fopen(path, "wb");
    if (!F.f) return fail(PTICM_ERR_IO, std::string("cannot write ") + path);
    F.put("PTICMCKP", 8);
    F.put_val<uint32_t>(kCkptVersion);
    F.put_val<uint32_t>(0);
    for (uint64_t v : ckpt_identity(c)) F.put_val<uint64_t>(v);
    F.put_val<uint64_t>((uint64_t)c->desc.n_pad);
    F.put_val<uint64_t>(c->steps_done);
    F.put_val<uint64_t>(c->attempts);
    F.put_val<int64_t>(c->nc);
    F.put(c->beta.data(), c->beta.size() * sizeof(double));
    const bool hist = c->d_hist.p != nullptr;
    F.put_val<uint64_t>(hist ? c->hist_from : 0);
    F.put_val<int64_t>(hist ? c->hist_lo : 0);
    F.put_val<int64_t>(hist ? c->hist_nbins : 0);
    int rc = PTICM_OK;
    if (!rc) rc = ckpt_dump(F, c->d_spins);
    if (!rc) rc = ckpt_dump(F, c->d_fields);
    if (!rc) rc = ckpt_dump(F, c->d_E);
    if (!rc) rc = ckpt_dump(F, c->d_bestE);
    if (!rc) rc = ckpt_dump(F, c->d_best_state);
    if (!rc) rc = ckpt_dump(F, c->d_flips);
    if (!rc) rc = ckpt_dump(F, c->d_bestSweep);
    if (!rc) rc = ckpt_dump(F, c->d_att);
    if (!rc) rc = ckpt_dump(F, c->d_succ);
    if (!rc) rc = ckpt_dump(F, c->d_slot);
    if (!rc) rc = ckpt_dump(F, c->d_order);
    if (!rc) rc = ckpt_dump(F, c->d_cursor);
    if (!rc && hist) rc = ckpt_dump(F, c->d_hist);
    if (!rc && hist) rc = ckpt_dump(F, c->d_obs);
    if (rc) return rc;
    if (!F.ok) return fail(PTICM_ERR_IO, std::string("short write to ") + path);
    return PTICM_OK;
}

int pticm_checkpoint_load(pticm_ctx* c, const char* path) {
    if (!c || !path) return fail(PTICM_ERR_INVALID, "null argument");
    CkptFile F;
    F.f = fopen(path, "rb");
    if (!F.f) return fail(PTICM_ERR_IO, std::string("cannot read ") + path);
    char magic[8] = {};
    F.get(magic, 8);
    const uint32_t version = F.get_val<uint32_t>();
    F.get_val<uint32_t>();
    if (!F.ok || memcmp(magic, "PTICMCKP", 8) != 0 || version != kCkptVersion)
        return fail(PTICM_ERR_INVALID, "not a PT-ICM checkpoint of this version");
    const std::vector<uint64_t> want = ckpt_identity(c);
    for (size_t k = 0; k < want.size(); k++)
        if (F.get_val<uint64_t>() != want[k] || !F.ok)
            return fail(PTICM_ERR_INVALID,
                        "checkpoint was written for another problem, ladder size or option set");
    if (int rc = configure(c, false)) return rc;
    if (F.get_val<uint64_t>() != (uint64_t)c->desc.n_pad)
        return fail(PTICM_ERR_INVALID, "checkpoint site padding differs");
    const uint64_t steps = F.get_val<uint64_t>(), attempts = F.get_val<uint64_t>();
    const int64_t nc = F.get_val<int64_t>();
    std::vector<double> beta((size_t)c->nt);
    F.get(beta.data(), beta.size() * sizeof(double));
    const uint64_t hist_from = F.get_val<uint64_t>();
    const int64_t hist_lo = F.get_val<int64_t>(), hist_nbins = F.get_val<int64_t>();
    if (!F.ok) return fail(PTICM_ERR_IO, "checkpoint header is truncated");
    if (int rc = pticm_set_ladder(c, beta.data(), (uint32_t)c->nt, (int32_t)nc)) return rc;
    if (hist_nbins > 0) {
        if (int rc = pticm_enable_energy_histograms(c, hist_from)) return rc;
        if (c->hist_lo != hist_lo || c->hist_nbins != hist_nbins)
            return fail(PTICM_ERR_INVALID, "checkpoint histogram range differs");
    }
    int rc = PTICM_OK;
    if (!rc) rc = ckpt_restore(F, c->d_spins, "spins");
    if (!rc) rc = ckpt_restore(F, c->d_fields, "fields");
    if (!rc) rc = ckpt_restore(F, c->d_E, "energies");
    if (!rc) rc = ckpt_restore(F, c->d_bestE, "best energies");
    if (!rc) rc = ckpt_restore(F, c->d_best_state, "best states");
    if (!rc) rc = ckpt_restore(F, c->d_flips, "flip counts");
    if (!rc) rc = ckpt_restore(F, c->d_bestSweep, "best sweeps");
    if (!rc) rc = ckpt_restore(F, c->d_att, "swap attempts");
    if (!rc) rc = ckpt_restore(F, c->d_succ, "swap successes");
    if (!rc) rc = ckpt_restore_permutation(F, c->d_slot, (size_t)c->R, "slot map");
    if (!rc) rc = ckpt_restore_permutation(F, c->d_order, (size_t)std::max(c->nt - 1, 0), "exchange order");
    if (!rc) rc = ckpt_restore(F, c->d_cursor, "exchange cursor");
    if (!rc && hist_nbins > 0) rc = ckpt_restore(F, c->d_hist, "histograms");
    if (!rc && hist_nbins > 0) rc = ckpt_restore(F, c->d_obs, "observables");
    if (rc) return rc;
    c->steps_done = steps;
    c->attempts = attempts;
    c->states_set = true;
    return PTICM_OK;
}

int pticm_philox_probe(const uint32_t* ctr, const uint32_t* key, uint32_t* out, int count) {
    if (!ctr || !key || !out || count <= 0) return fail(PTICM_ERR_INVALID, "invalid arguments");
    if (int rc = check_device()) return rc;
    DArr<uint4> dc, dout;
    DArr<uint2> dk;
    CK(dc.alloc(count));
    CK(dk.alloc(count));
    CK(dout.alloc(count));
    CK(cudaMemcpy(dc.p, ctr, (size_t)count * 16, cudaMemcpyHostToDevice));
    CK(cudaMemcpy(dk.p, key, (size_t)count * 8, cudaMemcpyHostToDevice));
    CK(launch_philox_probe(dc.p, dk.p, dout.p, count, nullptr));
    CK(cudaMemcpy(out, dout.p, (size_t)count * 16, cudaMemcpyDeviceToHost));
    return PTICM_OK;
}

}  // extern "C"
