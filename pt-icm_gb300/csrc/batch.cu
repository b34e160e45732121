// batch.cu -- many PT instances in one persistent engine launch
// (pticm_batch_*, include/pticm.h).
//
// Instances of different sizes share one cooperative launch of `lanes`
// co-resident blocks.  Instance i is split over g_i blocks of R/g_i replicas;
// the blocks of an instance meet at the instance's own group barrier.  Every
// block runs a list of jobs (instance, rank) sorted by one global key (the
// start time of the list schedule, then the instance index), so a block only
// ever waits for blocks that have finished every job ordered before: no
// cycle of waits can form while all blocks are resident.
//
// The autotuner runs a few PT steps at up to three group sizes per instance,
// reads each job's device time, and picks the g_i that minimise the
// makespan of the list schedule (longest-first onto the least-loaded lanes).
#include <cuda_runtime.h>

#include <algorithm>
#include <atomic>
#include <cfloat>
#include <cmath>
#include <memory>
#include <numeric>
#include <random>
#include <string>
#include <thread>
#include <vector>

#include "pticm.h"
#include "pticm_engine.h"
#include "problem_host.h"
#include "runtime_internal.h"

using namespace pticm;

namespace {

int bfail(int code, const std::string& m) {
    set_last_error(m);
    return code;
}

#define BCK(x)                                                                                       \
    do {                                                                                             \
        cudaError_t e_ = (x);                                                                        \
        if (e_ != cudaSuccess) return bfail(PTICM_ERR_CUDA, std::string(#x) + ": " + cudaGetErrorString(e_)); \
    } while (0)

constexpr double kLaunchTargetUs = 500000.0;   // aim: one launch ~0.5 s, a quarter of the 2 s wait limit

}  // namespace

struct pticm_batch {
    std::vector<HostProblem> P;
    long long ebound = -1;      // largest energy_bound over the instances, once
    pticm_opts o{};
    int count = 0, nt = 0, C = 0, R = 0, threads = 1024;
    std::vector<InstanceDesc> desc;
    std::vector<int> gmin;               // smallest group whose replicas fit a block
    std::vector<int> group;              // chosen group per instance
    std::vector<double> step_us;         // measured (or modelled) PT-step time per instance
    std::vector<double> beta;            // count * nt
    bool ladder_set = false, states_set = false, tuned = false;
    int lanes = 0, chunk = 1;
    double makespan_us = 0.0;            // predicted per PT step
    double step_ms_measured = 0.0;       // device time of one PT step of the current schedule (0: unknown)
    std::vector<int32_t> sched_measured; // the schedule step_ms_measured belongs to
    SmemPlan plan{};
    std::vector<int32_t> sched_off, sched;
    uint64_t steps_done = 0, attempts = 0, sites_total = 0, launches = 0;
    double last_ms = 0.0;
    uint64_t hist_from = 0;
    bool hist_on = false;
    std::vector<MhOutput> dos;           // multihistogram ln g per instance (pticm_batch_compute_logdos)
    double dos_estep = 0.0;
    cudaStream_t stream = nullptr;
    cudaEvent_t ev0 = nullptr, ev1 = nullptr;
    DArr<InstanceDesc> d_desc;
    DArr<int32_t> d_sched_off, d_sched, d_rep_inst, d_row, d_col, d_h;
    DArr<uint32_t> d_adj, d_thr, d_slot, d_order;
    DArr<double> d_beta;
    DArr<int8_t> d_spins, d_pub, d_best_state;
    DArr<int32_t> d_fields;
    DArr<long long> d_E, d_Epub, d_bestE;
    DArr<unsigned long long> d_flips, d_bestSweep, d_att, d_succ, d_mismatch, d_job_ns;
    DArr<unsigned int> d_hist, d_bar;
    DArr<int> d_abort;
    DArr<DevStatus> d_status;
    ~pticm_batch() {
        if (ev0) cudaEventDestroy(ev0);
        if (ev1) cudaEventDestroy(ev1);
        if (stream) cudaStreamDestroy(stream);
    }
};

namespace {

double model_step_us(const InstanceDesc& D, int g, int threads);

// ICM teams of an instance's blocks: one warp per pair for small instances,
// one block-wide team (pairs in sequence) from kBlockTeamSites sites on.
constexpr int kBlockTeamSites = 768;

int batch_teams(const InstanceDesc& D, int threads) {
    if (D.n_pad >= kBlockTeamSites) return 1;
    const int npairs = D.nc * (D.chains / 2);
    return std::max(1, std::min(threads / 32, std::max(1, npairs)));
}

// Shared-memory plan of the batch for the current groups: every instance
// unstaged first, ICM teams shrunk until the plan fits, then adjacency
// staging for every instance whose rows and edges fit what is left.
int plan_batch(pticm_batch* b, std::string& msg) {
    std::vector<InstanceDesc>& Ds = b->desc;
    std::vector<int> teams(b->count);
    for (int i = 0; i < b->count; i++) {
        Ds[i].group = b->group[i];
        Ds[i].rpc = b->R / b->group[i];
        teams[i] = batch_teams(Ds[i], b->threads);
    }
    auto dims_for = [&](long long stage_cap) {
        PlanDims d;
        for (int i = 0; i < b->count; i++) {
            const long long bytes = (long long)align16((uint64_t)(Ds[i].n + 1) * 4) + align16((uint64_t)Ds[i].nnz * 4);
            d.add(Ds[i], bytes <= stage_cap, teams[i]);
        }
        return d;
    };
    SmemPlan S = layout_plan(dims_for(-1));
    while (S.total > kSmemLimit) {
        // shrink the ICM teams of the instances with the largest scratch;
        // when every instance is down to one team, split the instance with
        // the most replica sites per block over more blocks
        uint64_t worst = 0;
        for (int i = 0; i < b->count; i++)
            worst = std::max(worst, (uint64_t)teams[i] * icm_team_bytes(Ds[i].n_pad));
        bool changed = false;
        for (int i = 0; i < b->count; i++)
            if (teams[i] > 1 && (uint64_t)teams[i] * icm_team_bytes(Ds[i].n_pad) == worst) {
                teams[i] = std::max(1, teams[i] / 2);
                changed = true;
            }
        if (!changed) {
            int big = -1;
            uint64_t sites = 0;
            for (int i = 0; i < b->count; i++) {
                const uint64_t si = (uint64_t)Ds[i].rpc * (uint64_t)Ds[i].n_pad;
                if (Ds[i].rpc > 1 && si > sites) { sites = si; big = i; }
            }
            if (big < 0) {
                msg = "the largest instance does not fit a block even with one replica per block";
                return PTICM_ERR_UNSUPPORTED;
            }
            int g = b->group[big] + 1;
            while (b->R % g) g++;
            b->group[big] = g;
            Ds[big].group = g;
            Ds[big].rpc = b->R / g;
            teams[big] = batch_teams(Ds[big], b->threads);
            if (!b->tuned) b->step_us[big] = model_step_us(Ds[big], g, b->threads);
        }
        S = layout_plan(dims_for(-1));
    }
    // largest staging size that still fits
    std::vector<long long> sizes;
    for (int i = 0; i < b->count; i++)
        sizes.push_back((long long)align16((uint64_t)(Ds[i].n + 1) * 4) + align16((uint64_t)Ds[i].nnz * 4));
    std::sort(sizes.begin(), sizes.end());
    sizes.erase(std::unique(sizes.begin(), sizes.end()), sizes.end());
    long long cap = -1;
    for (long long sz : sizes) {
        if (layout_plan(dims_for(sz)).total <= kSmemLimit) cap = sz;
        else break;
    }
    S = layout_plan(dims_for(cap));
    for (int i = 0; i < b->count; i++) {
        const long long bytes = (long long)align16((uint64_t)(Ds[i].n + 1) * 4) + align16((uint64_t)Ds[i].nnz * 4);
        Ds[i].stage = bytes <= cap ? 1 : 0;
        Ds[i].teams = teams[i];
    }
    b->plan = S;
    return PTICM_OK;
}

// Step-time model used before any measurement: a sweep costs about 2 ns per
// site-update per thread-slot plus 0.5 ns per edge, every phase has a fixed
// cost, a group barrier about 4 us.
double model_step_us(const InstanceDesc& D, int g, int threads) {
    const double rpc = (double)D.R / g;
    const double per_rep = (double)D.n * 2.0 + (double)D.nnz * 0.5;
    const double sweep = rpc * per_rep / threads * 1e-3 * 8.0 + 1.0 * D.ncolors;
    const double icm = D.nc > 0 ? (double)D.nc * (D.chains / 2) / g * ((double)D.n + D.nnz) * 0.02 * 1e-3 * 32 : 0.0;
    return 5.0 + sweep + icm + (g > 1 ? 4.0 : 0.0);
}

// List schedule: instances longest first, each onto the g lanes that are
// free earliest, starting when the last of them is free.
double build_schedule(pticm_batch* b) {
    const int L = b->lanes;
    std::vector<double> free(L, 0.0);
    struct Job { double start; int inst, rank; };
    std::vector<std::vector<Job>> jobs(L);
    std::vector<int> order(b->count);
    std::iota(order.begin(), order.end(), 0);
    std::stable_sort(order.begin(), order.end(), [&](int a, int c) {
        const double wa = b->step_us[a], wc = b->step_us[c];
        if (wa != wc) return wa > wc;
        return b->group[a] > b->group[c];
    });
    std::vector<int> lane(L);
    for (int i : order) {
        const int g = b->group[i];
        std::iota(lane.begin(), lane.end(), 0);
        std::partial_sort(lane.begin(), lane.begin() + g, lane.end(), [&](int x, int y) {
            if (free[x] != free[y]) return free[x] < free[y];
            return x < y;
        });
        double start = 0.0;
        for (int r = 0; r < g; r++) start = std::max(start, free[lane[r]]);
        for (int r = 0; r < g; r++) {
            jobs[lane[r]].push_back({start, i, r});
            free[lane[r]] = start + b->step_us[i];
        }
    }
    b->sched_off.assign(L + 1, 0);
    b->sched.clear();
    for (int l = 0; l < L; l++) {
        std::stable_sort(jobs[l].begin(), jobs[l].end(), [](const Job& x, const Job& y) {
            if (x.start != y.start) return x.start < y.start;
            return x.inst < y.inst;
        });
        for (const Job& j : jobs[l]) {
            b->sched.push_back(j.inst);
            b->sched.push_back(j.rank);
        }
        b->sched_off[l + 1] = (int32_t)(b->sched.size() / 2);
    }
    return *std::max_element(free.begin(), free.end());
}

// Plan, lanes, schedule and descriptors for the current groups and step
// times; uploads the descriptors and the schedule.
int configure_batch(pticm_batch* b) {
    std::string msg;
    if (int rc = plan_batch(b, msg)) return bfail(rc, msg);
    int dev = 0, sms = 0, per_sm = 0;
    BCK(cudaGetDevice(&dev));
    BCK(cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev));
    BCK(engine_max_blocks_per_sm(false, false, false, b->threads, b->plan.total, &per_sm));
    if (per_sm < 1) return bfail(PTICM_ERR_UNSUPPORTED, "the engine block does not fit on an SM");
    long long total_blocks = 0;
    int gmax = 0;
    for (int i = 0; i < b->count; i++) {
        total_blocks += b->group[i];
        gmax = std::max(gmax, b->group[i]);
    }
    b->lanes = (int)std::min<long long>((long long)per_sm * sms, total_blocks);
    if (gmax > b->lanes)
        return bfail(PTICM_ERR_UNSUPPORTED, "an instance needs more blocks than can be resident at once");
    b->makespan_us = build_schedule(b);
    // launches are sized from measured step times only (the model can be far
    // off): a schedule not measured yet starts with one-step launches
    if (b->sched != b->sched_measured) b->step_ms_measured = 0.0;
    b->chunk = b->step_ms_measured > 0
                   ? (int)std::max(1.0, std::min(65536.0, std::floor(kLaunchTargetUs / 1000.0 / b->step_ms_measured)))
                   : 1;
    for (int i = 0; i < b->count; i++) b->desc[i].first_block = 0;
    BCK(b->d_desc.upload(b->desc));
    BCK(b->d_sched_off.upload(b->sched_off));
    BCK(b->d_sched.upload(b->sched));
    return PTICM_OK;
}

EngineArgs batch_args(pticm_batch* b) {
    EngineArgs A{};
    A.desc = b->d_desc.p;
    A.sched_off = b->d_sched_off.p;
    A.sched = b->d_sched.p;
    A.n_inst = b->count;
    A.n_blocks = b->lanes;
    A.row = b->d_row.p;
    A.adj = b->d_adj.p;
    A.col = b->d_col.p;
    A.hpool = b->d_h.p;
    A.beta = b->d_beta.p;
    A.thr = b->d_thr.p;
    A.ptab = nullptr;
    A.perm = nullptr;
    A.spins = b->d_spins.p;
    A.fields = b->d_fields.p;
    A.energy = b->d_E.p;
    A.spins_pub = b->d_pub.p;
    A.spins_pub_half = (long long)b->d_spins.n;
    A.energy_pub = b->d_Epub.p;
    A.energy_pub_half = (long long)b->d_E.n;
    A.flips = b->d_flips.p;
    A.best_E = b->d_bestE.p;
    A.best_sweep = b->d_bestSweep.p;
    A.best_state = b->d_best_state.p;
    A.slot_rep = b->d_slot.p;
    A.xorder = b->d_order.p;
    A.xcursor = nullptr;
    A.attempts = b->d_att.p;
    A.successes = b->d_succ.p;
    A.bar = b->d_bar.p;
    if (b->ebound < 0) {
        b->ebound = 0;
        for (const HostProblem& P : b->P) b->ebound = std::max(b->ebound, energy_bound(P));
    }
    A.flag_barrier = b->ebound < (1ll << 31) ? 1 : 0;   // every energy fits the word's 32 bits
    A.abort_flag = b->d_abort.p;
    A.status = b->d_status.p;
    A.sweeps = (int)b->o.sweeps;
    A.seed = b->o.seed;
    A.sm = b->plan;
    A.prof = nullptr;
    A.job_ns = nullptr;
    A.hist = b->hist_on ? b->d_hist.p : nullptr;
    A.hist_from = b->hist_from;
    A.flags = (b->o.best_per_phase ? ENGINE_BEST_PER_PHASE : 0) | (b->o.exchange == 1 ? ENGINE_EXCHANGE_EVEN_ODD : 0);
    return A;
}

int batch_status(pticm_batch* b, const char* what) {
    DevStatus st{};
    BCK(cudaMemcpy(&st, b->d_status.p, sizeof(st), cudaMemcpyDeviceToHost));
    if (st.error)
        return bfail(PTICM_ERR_DEVICE, std::string(what) + ": device error " + std::to_string(st.error) + " at site " +
                                           std::to_string(st.where) + " (" + std::to_string(st.aux0) + ", " +
                                           std::to_string(st.aux1) + ")");
    return PTICM_OK;
}

// One launch of `steps` PT steps of every instance.
int batch_launch(pticm_batch* b, uint64_t step0, int steps, uint32_t phase_mask, unsigned long long* job_ns,
                 float* ms_out) {
    BCK(cudaMemsetAsync(b->d_bar.p, 0, b->d_bar.n * sizeof(unsigned), b->stream));
    BCK(cudaMemsetAsync(b->d_abort.p, 0, sizeof(int), b->stream));
    BCK(cudaMemsetAsync(b->d_status.p, 0, sizeof(DevStatus), b->stream));
    EngineArgs A = batch_args(b);
    A.step0 = step0;
    A.nsteps = steps;
    A.phase_mask = (int)phase_mask;
    A.job_ns = job_ns;
    BCK(cudaEventRecord(b->ev0, b->stream));
    BCK(launch_engine(A, b->threads, false, false, false, true, b->stream));
    BCK(cudaEventRecord(b->ev1, b->stream));
    BCK(cudaEventSynchronize(b->ev1));
    float ms = 0.f;
    BCK(cudaEventElapsedTime(&ms, b->ev0, b->ev1));
    if (ms_out) *ms_out = ms;
    return batch_status(b, "pticm_batch_run");
}

// Fresh bookkeeping after new spins (as the single-instance context).
int batch_reset_run_state(pticm_batch* b) {
    EngineArgs A = batch_args(b);
    const int total = (int)b->d_E.n;
    BCK(launch_recompute(A, b->d_rep_inst.p, total, 1, nullptr, nullptr, nullptr, b->stream));
    std::vector<long long> be(total, kNoBest);
    BCK(cudaMemcpyAsync(b->d_bestE.p, be.data(), be.size() * 8, cudaMemcpyHostToDevice, b->stream));
    BCK(cudaMemcpyAsync(b->d_best_state.p, b->d_spins.p, b->d_spins.n, cudaMemcpyDeviceToDevice, b->stream));
    BCK(cudaMemsetAsync(b->d_bestSweep.p, 0, total * 8, b->stream));
    BCK(cudaMemsetAsync(b->d_flips.p, 0, total * 8, b->stream));
    BCK(cudaMemsetAsync(b->d_att.p, 0, total * 8, b->stream));
    BCK(cudaMemsetAsync(b->d_succ.p, 0, total * 8, b->stream));
    std::vector<uint32_t> slot(total), order(total, 0);
    std::mt19937_64 g(b->o.seed ^ 0x6F72646572ull);
    for (int i = 0; i < b->count; i++) {
        const InstanceDesc& D = b->desc[i];
        for (int r = 0; r < D.R; r++) slot[D.rep_off + r] = (uint32_t)r;
        for (int k = 0; k + 1 < D.nt; k++) order[D.rep_off + k] = (uint32_t)k;
        if (D.nt > 2) std::shuffle(order.begin() + D.rep_off, order.begin() + D.rep_off + (D.nt - 1), g);
    }
    BCK(cudaMemcpyAsync(b->d_slot.p, slot.data(), slot.size() * 4, cudaMemcpyHostToDevice, b->stream));
    BCK(cudaMemcpyAsync(b->d_order.p, order.data(), order.size() * 4, cudaMemcpyHostToDevice, b->stream));
    BCK(cudaStreamSynchronize(b->stream));
    b->steps_done = 0;
    b->attempts = 0;
    b->states_set = true;
    return PTICM_OK;
}

// Device copy of every pool a run changes (for the autotuner's trial runs).
struct Snapshot {
    DArr<int8_t> spins, best_state;
    DArr<int32_t> fields;
    DArr<long long> E, bestE;
    DArr<unsigned long long> flips, bestSweep, att, succ;
    DArr<uint32_t> slot, order;
    DArr<unsigned int> hist;
};

template <typename T>
cudaError_t dcopy(DArr<T>& dst, const DArr<T>& src, cudaStream_t st) {
    if (dst.n != src.n) {
        cudaError_t e = dst.alloc(src.n);
        if (e != cudaSuccess) return e;
    }
    if (!src.n) return cudaSuccess;
    return cudaMemcpyAsync(dst.p, src.p, src.n * sizeof(T), cudaMemcpyDeviceToDevice, st);
}

int snapshot(pticm_batch* b, Snapshot& s, bool save) {
    cudaStream_t st = b->stream;
    if (save) {
        BCK(dcopy(s.spins, b->d_spins, st)); BCK(dcopy(s.best_state, b->d_best_state, st));
        BCK(dcopy(s.fields, b->d_fields, st)); BCK(dcopy(s.E, b->d_E, st)); BCK(dcopy(s.bestE, b->d_bestE, st));
        BCK(dcopy(s.flips, b->d_flips, st)); BCK(dcopy(s.bestSweep, b->d_bestSweep, st));
        BCK(dcopy(s.att, b->d_att, st)); BCK(dcopy(s.succ, b->d_succ, st));
        BCK(dcopy(s.slot, b->d_slot, st)); BCK(dcopy(s.order, b->d_order, st)); BCK(dcopy(s.hist, b->d_hist, st));
    } else {
        BCK(dcopy(b->d_spins, s.spins, st)); BCK(dcopy(b->d_best_state, s.best_state, st));
        BCK(dcopy(b->d_fields, s.fields, st)); BCK(dcopy(b->d_E, s.E, st)); BCK(dcopy(b->d_bestE, s.bestE, st));
        BCK(dcopy(b->d_flips, s.flips, st)); BCK(dcopy(b->d_bestSweep, s.bestSweep, st));
        BCK(dcopy(b->d_att, s.att, st)); BCK(dcopy(b->d_succ, s.succ, st));
        BCK(dcopy(b->d_slot, s.slot, st)); BCK(dcopy(b->d_order, s.order, st)); BCK(dcopy(b->d_hist, s.hist, st));
    }
    BCK(cudaStreamSynchronize(st));
    return PTICM_OK;
}

}  // namespace

extern "C" {

int pticm_batch_create(const pticm_problem* const* problems, uint32_t count, const pticm_opts* o,
                       pticm_batch** out) {
    if (!problems || !o || !out || count == 0) return bfail(PTICM_ERR_INVALID, "null argument or empty batch");
    if (count > 65535) return bfail(PTICM_ERR_INVALID, "at most 65535 instances per batch");
    if (o->nt < 2) return bfail(PTICM_ERR_INVALID, "at least two temperatures are needed");
    if (o->chains < 1 || o->chains > 16) return bfail(PTICM_ERR_INVALID, "chains must be in [1, 16]");
    if (o->icm && (o->chains % 2)) return bfail(PTICM_ERR_INVALID, "ICM pairs chains: use an even chain count");
    if (o->sweeps < 1 || o->exchange > 1 || o->icm_algo > 3) return bfail(PTICM_ERR_INVALID, "invalid options");
    if (o->block_threads && (o->block_threads % 32 || o->block_threads > (uint32_t)kNarrowThreads))
        return bfail(PTICM_ERR_INVALID, "block_threads must be a multiple of 32, at most 512");
    int ndev = 0;
    if (cudaGetDeviceCount(&ndev) != cudaSuccess || ndev == 0)
        return bfail(PTICM_ERR_NODEVICE, "no CUDA device is available; the PT-ICM engine has no CPU path");
    for (uint32_t i = 0; i < count; i++)
        if (!problems[i]) return bfail(PTICM_ERR_INVALID, "null problem in the batch");
    auto b = std::make_unique<pticm_batch>();
    b->o = *o;
    b->count = (int)count;
    b->nt = (int)o->nt;
    b->C = (int)o->chains;
    b->R = b->nt * b->C;
    b->threads = o->block_threads ? (int)o->block_threads : kNarrowThreads;
    b->P.reserve(count);
    for (uint32_t i = 0; i < count; i++) b->P.push_back(problem_host(problems[i]));
    // pools
    std::vector<int32_t> row, col, h, rep_inst;
    std::vector<uint32_t> adj;
    int64_t spin_total = 0, rep_total = 0, thr_total = 0;
    b->desc.resize(count);
    for (uint32_t i = 0; i < count; i++) {
        const HostProblem& P = b->P[i];
        InstanceDesc& D = b->desc[i];
        D.n = (int32_t)P.n;
        D.n_pad = pad16(P.n);
        D.nnz = (int32_t)P.dadj.size();
        D.ncolors = P.ncolors;
        D.kmax = P.kmax;
        D.nt = b->nt;
        D.chains = b->C;
        D.R = b->R;
        D.has_h = P.has_h ? 1 : 0;
        D.inst_id = (int32_t)i;
        D.icm_algo = engine_flags(P, *o) & ENGINE_ICM_MASK;
        // every segment starts on 16 bytes: the adjacency is staged by bulk
        // copies, which need 16-byte aligned global addresses
        D.row_off = (int64_t)row.size();
        row.insert(row.end(), P.drow.begin(), P.drow.end());
        row.resize((row.size() + 3) & ~size_t(3), 0);
        D.adj_off = (int64_t)adj.size();
        adj.insert(adj.end(), P.dadj.begin(), P.dadj.end());
        adj.resize((adj.size() + 3) & ~size_t(3), 0u);
        D.col_off = (int64_t)col.size();
        col.insert(col.end(), P.color_off.begin(), P.color_off.end());
        col.resize((col.size() + 3) & ~size_t(3), 0);
        D.h_off = (int64_t)h.size();
        h.insert(h.end(), P.dh.begin(), P.dh.end());
        h.resize((h.size() + 3) & ~size_t(3), 0);
        D.beta_off = (int64_t)i * b->nt;
        D.thr_off = thr_total;
        thr_total += (int64_t)b->nt * (P.kmax + 1);
        D.rep_off = rep_total;
        rep_total += b->R;
        D.spin_off = spin_total;
        spin_total += (int64_t)b->R * D.n_pad;
        for (int r = 0; r < b->R; r++) rep_inst.push_back((int32_t)i);
        b->sites_total += (uint64_t)P.n * (uint64_t)b->R;
    }
    BCK(cudaStreamCreateWithFlags(&b->stream, cudaStreamNonBlocking));
    BCK(cudaEventCreate(&b->ev0));
    BCK(cudaEventCreate(&b->ev1));
    BCK(b->d_row.upload(row, 4));
    BCK(b->d_adj.upload(adj, 4));
    BCK(b->d_col.upload(col, 4));
    BCK(b->d_h.upload(h, 4));
    BCK(b->d_rep_inst.upload(rep_inst));
    BCK(b->d_spins.alloc(spin_total));
    BCK(b->d_fields.alloc(spin_total));
    BCK(b->d_best_state.alloc(spin_total));
    BCK(b->d_pub.alloc(2 * spin_total));
    BCK(b->d_E.alloc(rep_total));
    BCK(b->d_Epub.alloc(2 * rep_total * kPubStride));
    BCK(b->d_bestE.alloc(rep_total));
    BCK(b->d_flips.alloc(rep_total));
    BCK(b->d_bestSweep.alloc(rep_total));
    BCK(b->d_att.alloc(rep_total));
    BCK(b->d_succ.alloc(rep_total));
    BCK(b->d_slot.alloc(rep_total));
    BCK(b->d_order.alloc(rep_total));
    BCK(b->d_thr.alloc(thr_total + 4));
    BCK(b->d_beta.alloc((size_t)count * b->nt));
    BCK(b->d_bar.alloc(2 * (size_t)count));
    BCK(b->d_abort.alloc(1));
    BCK(b->d_status.alloc(1));
    BCK(b->d_mismatch.alloc(1));
    // smallest group per instance: replicas of a block fit shared memory
    // (unstaged, one ICM team) on their own
    b->gmin.assign(count, 0);
    b->group.assign(count, 0);
    b->step_us.assign(count, 0.0);
    for (uint32_t i = 0; i < count; i++) {
        InstanceDesc D = b->desc[i];
        for (int g = 1; g <= b->R; g++) {
            if (b->R % g) continue;
            D.rpc = b->R / g;
            D.group = g;
            if (make_plan(D, false, 1, b->threads, false).total <= kSmemLimit) {
                b->gmin[i] = g;
                break;
            }
        }
        if (!b->gmin[i])
            return bfail(PTICM_ERR_UNSUPPORTED, "instance " + std::to_string(i) + " does not fit a block even with one replica");
        int g = b->gmin[i];
        if (o->replicas_per_block) {
            if (b->R % (int)o->replicas_per_block) return bfail(PTICM_ERR_INVALID, "replicas_per_block must divide nt*chains");
            g = std::max(g, b->R / (int)o->replicas_per_block);
        }
        b->group[i] = g;
        b->step_us[i] = model_step_us(b->desc[i], g, b->threads);
    }
    *out = b.release();
    return PTICM_OK;
}

void pticm_batch_destroy(pticm_batch* b) { delete b; }

int pticm_batch_set_ladders(pticm_batch* b, const double* beta, uint32_t nt, int32_t nc) {
    if (!b || !beta) return bfail(PTICM_ERR_INVALID, "null argument");
    if ((int)nt != b->nt) return bfail(PTICM_ERR_INVALID, "ladder length differs from the batch's nt");
    for (size_t k = 0; k < (size_t)b->count * nt; k++)
        if (!std::isfinite(beta[k])) return bfail(PTICM_ERR_INVALID, "non-finite inverse temperature");
    b->beta.assign(beta, beta + (size_t)b->count * nt);
    std::vector<uint32_t> thr_all;
    for (int i = 0; i < b->count; i++) {
        std::vector<uint32_t> thr;
        std::vector<double> ptab;
        b->desc[i].nc = ladder_tables(b->P[i], beta + (size_t)i * nt, (int)nt, nc, b->o.icm != 0, b->C, thr, ptab);
        thr_all.insert(thr_all.end(), thr.begin(), thr.end());
        b->step_us[i] = b->tuned ? b->step_us[i] : model_step_us(b->desc[i], b->group[i], b->threads);
    }
    BCK(b->d_beta.upload(b->beta));
    BCK(b->d_thr.upload(thr_all, 4));
    b->ladder_set = true;
    return PTICM_OK;
}

int pticm_batch_init_states(pticm_batch* b, uint64_t seed) {
    if (!b) return bfail(PTICM_ERR_INVALID, "null argument");
    if (int rc = configure_batch(b)) return rc;
    EngineArgs A = batch_args(b);
    BCK(launch_init_spins(A, b->d_rep_inst.p, (int)b->d_E.n, seed, b->stream));
    return batch_reset_run_state(b);
}

int pticm_batch_run(pticm_batch* b, uint64_t pt_steps, uint32_t phase_mask) {
    if (!b) return bfail(PTICM_ERR_INVALID, "null argument");
    if (!b->ladder_set) return bfail(PTICM_ERR_INVALID, "set the ladders before running");
    if (!b->states_set) return bfail(PTICM_ERR_INVALID, "initialise the replica states before running");
    if (phase_mask == 0 || phase_mask > 7) return bfail(PTICM_ERR_INVALID, "phase_mask must be in 1..7");
    if (int rc = configure_batch(b)) return rc;
    b->dos.clear();
    b->last_ms = 0.0;
    uint64_t left = pt_steps;
    while (left > 0) {
        const int chunk = (int)std::min<uint64_t>(left, (uint64_t)b->chunk);
        float ms = 0.f;
        if (int rc = batch_launch(b, b->steps_done, chunk, phase_mask, nullptr, &ms)) return rc;
        b->launches++;
        if (phase_mask == 7u) {
            b->step_ms_measured = std::max((double)ms / chunk, 1e-6);
            b->sched_measured = b->sched;
            b->chunk = (int)std::max(1.0, std::min(65536.0, std::floor(kLaunchTargetUs / 1000.0 / b->step_ms_measured)));
        }
        b->last_ms += ms;
        b->steps_done += (uint64_t)chunk;
        if (phase_mask & PHASE_SWEEP) b->attempts += (uint64_t)chunk * b->o.sweeps * b->sites_total;
        left -= (uint64_t)chunk;
    }
    return PTICM_OK;
}

int pticm_batch_autotune(pticm_batch* b, uint32_t trial_steps) {
    if (!b) return bfail(PTICM_ERR_INVALID, "null argument");
    if (!b->ladder_set || !b->states_set) return bfail(PTICM_ERR_INVALID, "set the ladders and states first");
    if (trial_steps < 3) return bfail(PTICM_ERR_INVALID, "the autotuner needs at least 3 trial steps");
    Snapshot snap;
    if (int rc = snapshot(b, snap, true)) return rc;
    // up to three group sizes per instance: g_min, then the next divisors of R
    // at or above 2 g_min and 4 g_min
    std::vector<std::vector<int>> cand(b->count);
    for (int i = 0; i < b->count; i++) {
        int want = b->gmin[i];
        for (int t = 0; t < 3; t++) {
            int g = want;
            while (g <= b->R && b->R % g) g++;
            if (g > b->R) break;
            if (cand[i].empty() || cand[i].back() != g) cand[i].push_back(g);
            want = 2 * g;
        }
    }
    // measured step time per instance and group actually run (the planner
    // may raise a group so that the batch's shared-memory plan fits)
    std::vector<std::vector<int>> mg(b->count);
    std::vector<std::vector<double>> meas(b->count);
    const std::vector<int> keep_group = b->group;
    for (int t = 0; t < 3; t++) {
        for (int i = 0; i < b->count; i++) {
            b->group[i] = cand[i][std::min<size_t>(t, cand[i].size() - 1)];
            b->step_us[i] = model_step_us(b->desc[i], b->group[i], b->threads);
        }
        if (int rc = configure_batch(b)) {
            b->group = keep_group;
            return rc;
        }
        DArr<unsigned long long> job_ns;
        BCK(job_ns.alloc(b->sched.size() / 2));
        // a two-step launch sizes the trial so that it stays near the launch target
        float ms = 0.f;
        if (int rc = batch_launch(b, b->steps_done, 2, PHASE_SWEEP | PHASE_EXCHANGE | PHASE_ICM, nullptr, &ms))
            return rc;
        const int steps_t = (int)std::max(3.0, std::min((double)trial_steps, std::floor(kLaunchTargetUs / 1000.0 / std::max(ms / 2.0, 1e-6))));
        if (int rc = batch_launch(b, b->steps_done, steps_t, PHASE_SWEEP | PHASE_EXCHANGE | PHASE_ICM, job_ns.p, &ms))
            return rc;
        std::vector<unsigned long long> ns;
        BCK(job_ns.download(ns));
        std::vector<double> worst(b->count, 0.0);
        for (size_t j = 0; j < ns.size(); j++) {
            const int inst = b->sched[2 * j];
            worst[inst] = std::max(worst[inst], (double)ns[j] * 1e-3 / (steps_t - 1));
        }
        for (int i = 0; i < b->count; i++)
            if (std::find(mg[i].begin(), mg[i].end(), b->group[i]) == mg[i].end()) {
                mg[i].push_back(b->group[i]);
                meas[i].push_back(worst[i]);
            }
        if (int rc = snapshot(b, snap, false)) return rc;
    }
    // sort each instance's measurements by group
    for (int i = 0; i < b->count; i++) {
        std::vector<int> ord(mg[i].size());
        std::iota(ord.begin(), ord.end(), 0);
        std::sort(ord.begin(), ord.end(), [&](int x, int y) { return mg[i][x] < mg[i][y]; });
        std::vector<int> g2;
        std::vector<double> m2;
        for (int k : ord) { g2.push_back(mg[i][k]); m2.push_back(meas[i][k]); }
        mg[i] = g2;
        meas[i] = m2;
    }
    cand = mg;
    // choose: most efficient group (least block-time g*t) first, then split
    // the instances that are longer than the average lane load
    std::vector<int> pick(b->count);
    double load = 0.0;
    for (int i = 0; i < b->count; i++) {
        int best = 0;
        for (size_t k = 1; k < meas[i].size(); k++)
            if (cand[i][k] * meas[i][k] < cand[i][best] * meas[i][best]) best = (int)k;
        pick[i] = best;
        load += cand[i][best] * meas[i][best];
    }
    int dev = 0, sms = 0;
    BCK(cudaGetDevice(&dev));
    BCK(cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev));
    for (int round = 0; round < 4 * b->count; round++) {
        const double avg = load / std::max(1, std::min(b->lanes, sms));
        int worst = -1;
        double wt = 0.0;
        for (int i = 0; i < b->count; i++)
            if (meas[i][pick[i]] > wt) { wt = meas[i][pick[i]]; worst = i; }
        if (worst < 0 || wt <= avg) break;
        // a larger group with a shorter step?
        int next = -1;
        for (size_t k = pick[worst] + 1; k < meas[worst].size(); k++)
            if (meas[worst][k] < wt) { next = (int)k; break; }
        if (next < 0) break;
        load += cand[worst][next] * meas[worst][next] - cand[worst][pick[worst]] * meas[worst][pick[worst]];
        pick[worst] = next;
    }
    for (int i = 0; i < b->count; i++) {
        b->group[i] = cand[i][pick[i]];
        b->step_us[i] = meas[i][pick[i]];
    }
    b->tuned = true;
    return configure_batch(b);
}

int pticm_batch_get_info(pticm_batch* b, pticm_batch_info* info) {
    if (!b || !info) return bfail(PTICM_ERR_INVALID, "null argument");
    info->count = (uint32_t)b->count;
    info->lanes = (uint32_t)b->lanes;
    info->chunk = (uint32_t)b->chunk;
    info->jobs = (uint32_t)(b->sched.size() / 2);
    info->smem_bytes = b->plan.total;
    info->threads = (uint32_t)b->threads;
    info->tuned = b->tuned ? 1 : 0;
    info->makespan_us = b->makespan_us;
    info->pt_steps = b->steps_done;
    info->attempts = b->attempts;
    info->last_run_ms = b->last_ms;
    info->launches = b->launches;
    return PTICM_OK;
}

int pticm_batch_get_groups(pticm_batch* b, uint32_t* group, double* step_us, int32_t* staged, int32_t* teams) {
    if (!b) return bfail(PTICM_ERR_INVALID, "null argument");
    for (int i = 0; i < b->count; i++) {
        if (group) group[i] = (uint32_t)b->group[i];
        if (step_us) step_us[i] = b->step_us[i];
        if (staged) staged[i] = b->desc[i].stage;
        if (teams) teams[i] = b->desc[i].teams;
    }
    return PTICM_OK;
}

int pticm_batch_get_best(pticm_batch* b, double* energy, uint64_t* flips) {
    if (!b) return bfail(PTICM_ERR_INVALID, "null argument");
    BCK(cudaStreamSynchronize(b->stream));
    std::vector<long long> be;
    std::vector<unsigned long long> fl;
    BCK(b->d_bestE.download(be));
    BCK(b->d_flips.download(fl));
    for (int i = 0; i < b->count; i++) {
        const InstanceDesc& D = b->desc[i];
        long long best = kNoBest;
        unsigned long long f = 0;
        for (int r = 0; r < D.R; r++) {
            best = std::min(best, be[D.rep_off + r]);
            f += fl[D.rep_off + r];
        }
        if (energy) energy[i] = best == kNoBest ? DBL_MAX : (double)best;
        if (flips) flips[i] = f;
    }
    return PTICM_OK;
}

int pticm_batch_get_best_state(pticm_batch* b, uint32_t inst, uint8_t* state) {
    if (!b || !state || (int)inst >= b->count) return bfail(PTICM_ERR_INVALID, "invalid arguments");
    BCK(cudaStreamSynchronize(b->stream));
    const InstanceDesc& D = b->desc[inst];
    std::vector<long long> be(D.R);
    BCK(cudaMemcpy(be.data(), b->d_bestE.p + D.rep_off, D.R * 8, cudaMemcpyDeviceToHost));
    int bi = -1;
    long long best = kNoBest;
    for (int r = 0; r < D.R; r++)
        if (be[r] < best) { best = be[r]; bi = r; }
    std::vector<int8_t> row(D.n_pad, 1);
    if (bi >= 0)
        BCK(cudaMemcpy(row.data(), b->d_best_state.p + D.spin_off + (int64_t)bi * D.n_pad, D.n_pad,
                       cudaMemcpyDeviceToHost));
    const HostProblem& P = b->P[inst];
    for (int i = 0; i < D.n; i++) state[P.perm[i]] = row[i] > 0 ? 1 : 0;
    return PTICM_OK;
}

int pticm_batch_get_swap_stats(pticm_batch* b, uint32_t inst, uint64_t* attempts, uint64_t* successes) {
    if (!b || (int)inst >= b->count) return bfail(PTICM_ERR_INVALID, "invalid arguments");
    BCK(cudaStreamSynchronize(b->stream));
    const InstanceDesc& D = b->desc[inst];
    std::vector<unsigned long long> a(D.R), s(D.R);
    BCK(cudaMemcpy(a.data(), b->d_att.p + D.rep_off, D.R * 8, cudaMemcpyDeviceToHost));
    BCK(cudaMemcpy(s.data(), b->d_succ.p + D.rep_off, D.R * 8, cudaMemcpyDeviceToHost));
    for (int k = 0; k < D.R; k++) {
        if (attempts) attempts[k] = a[k];
        if (successes) successes[k] = s[k];
    }
    return PTICM_OK;
}

int pticm_batch_get_energies(pticm_batch* b, uint32_t inst, int64_t* energy, uint32_t* slot_to_replica) {
    if (!b || (int)inst >= b->count) return bfail(PTICM_ERR_INVALID, "invalid arguments");
    BCK(cudaStreamSynchronize(b->stream));
    const InstanceDesc& D = b->desc[inst];
    if (energy) BCK(cudaMemcpy(energy, b->d_E.p + D.rep_off, D.R * 8, cudaMemcpyDeviceToHost));
    if (slot_to_replica) BCK(cudaMemcpy(slot_to_replica, b->d_slot.p + D.rep_off, D.R * 4, cudaMemcpyDeviceToHost));
    return PTICM_OK;
}

int pticm_batch_verify(pticm_batch* b, uint64_t* mismatches) {
    if (!b || !mismatches) return bfail(PTICM_ERR_INVALID, "null argument");
    if (!b->states_set) return bfail(PTICM_ERR_INVALID, "no states yet");
    BCK(cudaMemsetAsync(b->d_mismatch.p, 0, sizeof(unsigned long long), b->stream));
    EngineArgs A = batch_args(b);
    BCK(launch_recompute(A, b->d_rep_inst.p, (int)b->d_E.n, 0, b->d_mismatch.p, nullptr, nullptr, b->stream));
    unsigned long long mm = 0;
    BCK(cudaMemcpyAsync(&mm, b->d_mismatch.p, sizeof(mm), cudaMemcpyDeviceToHost, b->stream));
    BCK(cudaStreamSynchronize(b->stream));
    *mismatches = mm;
    return PTICM_OK;
}

int pticm_batch_enable_energy_histograms(pticm_batch* b, uint64_t from_step) {
    if (!b) return bfail(PTICM_ERR_INVALID, "null argument");
    int64_t off = 0;
    for (int i = 0; i < b->count; i++) {
        const long long w = energy_bound(b->P[i]);
        b->desc[i].hist_lo = -w;
        b->desc[i].hist_nbins = w + 1;
        b->desc[i].hist_off = off;
        off += (int64_t)b->R * (w + 1);
    }
    if ((uint64_t)off > (1ull << 34)) return bfail(PTICM_ERR_UNSUPPORTED, "energy histograms of the batch exceed 64 GB");
    BCK(b->d_hist.alloc((size_t)off));
    b->hist_from = from_step;
    b->hist_on = true;
    return PTICM_OK;
}

int pticm_batch_get_energy_histograms(pticm_batch* b, uint32_t inst, uint32_t* hist, int64_t* e_lo,
                                      uint64_t* nbins) {
    if (!b || (int)inst >= b->count) return bfail(PTICM_ERR_INVALID, "invalid arguments");
    if (!b->hist_on) return bfail(PTICM_ERR_INVALID, "energy histograms are not enabled");
    const InstanceDesc& D = b->desc[inst];
    if (e_lo) *e_lo = D.hist_lo;
    if (nbins) *nbins = (uint64_t)D.hist_nbins;
    if (hist) {
        BCK(cudaStreamSynchronize(b->stream));
        BCK(cudaMemcpy(hist, b->d_hist.p + D.hist_off, (size_t)D.R * D.hist_nbins * 4, cudaMemcpyDeviceToHost));
    }
    return PTICM_OK;
}

int pticm_batch_compute_logdos(pticm_batch* b, double estep) {
    if (!b || !(estep > 0)) return bfail(PTICM_ERR_INVALID, "invalid arguments");
    if (!b->hist_on) return bfail(PTICM_ERR_INVALID, "energy histograms are not enabled");
    BCK(cudaStreamSynchronize(b->stream));
    std::vector<MhInput> in(b->count);
    std::vector<int> rc(b->count, PTICM_OK);
    std::vector<std::string> msg(b->count);
    std::atomic<int> next{0};
    int dev = 0;
    BCK(cudaGetDevice(&dev));
    auto work = [&]() {
        cudaSetDevice(dev);
        std::vector<unsigned> rows;
        for (int i = next++; i < b->count; i = next++) {
            const InstanceDesc& D = b->desc[i];
            rows.resize((size_t)D.R * (size_t)D.hist_nbins);
            if (cudaMemcpy(rows.data(), b->d_hist.p + D.hist_off, rows.size() * 4, cudaMemcpyDeviceToHost) != cudaSuccess) {
                rc[i] = PTICM_ERR_CUDA;
                continue;
            }
            rc[i] = compact_slot_hist(rows.data(), D.nt, D.chains, D.hist_nbins, D.hist_lo,
                                      b->beta.data() + (size_t)i * b->nt, estep, in[i]);
        }
    };
    const int nthreads = (int)std::max(1u, std::min(16u, std::thread::hardware_concurrency()));
    std::vector<std::thread> pool;
    for (int t = 0; t < nthreads; t++) pool.emplace_back(work);
    for (auto& t : pool) t.join();
    for (int i = 0; i < b->count; i++)
        if (rc[i]) return bfail(rc[i], "instance " + std::to_string(i) + ": pilot histograms unusable");
    std::vector<const MhInput*> ptrs;
    for (auto& x : in) ptrs.push_back(&x);
    if (int r = mhist_dos_multi(ptrs, b->dos)) return r;
    b->dos_estep = estep;
    return PTICM_OK;
}

int pticm_batch_logdos(pticm_batch* b, uint32_t inst, double estep, double* logdos, uint64_t cap, uint64_t* nbins,
                       double* min_emin, uint64_t* iterations) {
    if (!b || (int)inst >= b->count || !nbins || !(estep > 0)) return bfail(PTICM_ERR_INVALID, "invalid arguments");
    if (!b->hist_on) return bfail(PTICM_ERR_INVALID, "energy histograms are not enabled");
    std::vector<double> dos, z;
    double me = 0.0;
    uint64_t it = 0;
    if (b->dos_estep == estep && (int)b->dos.size() == b->count) {
        dos = b->dos[inst].logdos;
        me = b->dos[inst].min_emin;
        it = b->dos[inst].iters;
    } else {
        BCK(cudaStreamSynchronize(b->stream));
        const InstanceDesc& D = b->desc[inst];
        std::vector<unsigned> rows((size_t)D.R * (size_t)D.hist_nbins);
        BCK(cudaMemcpy(rows.data(), b->d_hist.p + D.hist_off, rows.size() * 4, cudaMemcpyDeviceToHost));
        if (int rc = slot_hist_dos(rows.data(), D.nt, D.chains, D.hist_nbins, D.hist_lo,
                                   b->beta.data() + (size_t)inst * b->nt, estep, dos, z, me, it))
            return rc;
    }
    *nbins = dos.size();
    if (min_emin) *min_emin = me;
    if (iterations) *iterations = it;
    if (logdos) {
        if (cap < dos.size()) return bfail(PTICM_ERR_INVALID, "logdos buffer too small");
        std::copy(dos.begin(), dos.end(), logdos);
    }
    return PTICM_OK;
}

}  // extern "C"
