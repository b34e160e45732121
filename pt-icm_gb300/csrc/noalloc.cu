// noalloc.cu -- a PT-ICM run that allocates no device memory.
//
// Some callers cannot call cudaMalloc: code that runs inside a host framework
// which owns every device allocation (a pool or arena it hands out), or that
// must not trigger the implicit device synchronisation cudaMalloc/cudaFree
// can cause.  pticm_run_noalloc serves them: the caller passes its own device
// buffers for the inputs (initial spins, optional slot map and pair order)
// and the outputs (final spins, energies, exchange counts, best states); all
// working memory of the run -- the graph in the engine's layout, fields,
// published copies, barrier words and the error record -- lives in one
// file-scope __device__ array of PTICM_NOALLOC_SCRATCH_BYTES.  Every GPU that
// loads this library holds that array until the process exits.
//
// The first call on a device resolves the array's device address with
// cudaGetSymbolAddress (host code must never use the symbol itself as a
// pointer); make that first call before any stream capture.  All calls share
// the array and it keeps the last call's contents, so everything a run needs
// zeroed is cleared at the start of each call, and calls that overlap on the
// GPU (different streams, or different host threads) race on it.
#include <cuda_runtime.h>

#include <algorithm>
#include <cmath>
#include <cstring>
#include <mutex>
#include <string>
#include <vector>

#include "pticm.h"
#include "pticm_device.cuh"
#include "pticm_engine.h"
#include "problem_host.h"
#include "runtime_internal.h"

namespace pticm {

static __device__ __align__(256) unsigned char g_noalloc_scratch[PTICM_NOALLOC_SCRATCH_BYTES];

namespace {

std::mutex g_setup_mutex;
void* g_scratch_addr[256] = {nullptr};

int noalloc_fail(int code, const std::string& m) {
    set_last_error(m);
    return code;
}

#define NA_CK(x)                                                                                          \
    do {                                                                                                  \
        cudaError_t e_ = (x);                                                                             \
        if (e_ != cudaSuccess) return noalloc_fail(PTICM_ERR_CUDA, std::string(#x) + ": " + cudaGetErrorString(e_)); \
    } while (0)

// Device address of the scratch array on the current device, resolved once.
int scratch_address(void** out) {
    int dev = 0;
    NA_CK(cudaGetDevice(&dev));
    if (dev < 0 || dev >= 256) return noalloc_fail(PTICM_ERR_INVALID, "device index out of range");
    std::lock_guard<std::mutex> lock(g_setup_mutex);
    if (!g_scratch_addr[dev]) {
        void* p = nullptr;
        NA_CK(cudaGetSymbolAddress(&p, g_noalloc_scratch));
        g_scratch_addr[dev] = p;
    }
    *out = g_scratch_addr[dev];
    return PTICM_OK;
}

__global__ void import_spins(const uint8_t* in, int8_t* spins, const int32_t* perm, int n, int n_pad, int R) {
    const long long total = (long long)R * n_pad;
    for (long long x = blockIdx.x * (long long)blockDim.x + threadIdx.x; x < total; x += (long long)gridDim.x * blockDim.x) {
        const int r = (int)(x / n_pad), i = (int)(x - (long long)r * n_pad);
        spins[x] = (i < n) ? (in[(long long)r * n + perm[i]] ? 1 : -1) : 1;
    }
}

__global__ void export_spins(const int8_t* spins, uint8_t* out, const int32_t* perm, int n, int n_pad, int R) {
    const long long total = (long long)R * n;
    for (long long x = blockIdx.x * (long long)blockDim.x + threadIdx.x; x < total; x += (long long)gridDim.x * blockDim.x) {
        const int r = (int)(x / n), i = (int)(x - (long long)r * n);
        out[(long long)r * n + perm[i]] = spins[(long long)r * n_pad + i] > 0 ? 1 : 0;
    }
}

// The caller's slot map and pair order are used as indices by the engine:
// check that each is a permutation (slot: of 0..R-1, order: of 0..nt-2)
// before it runs.  `seen` holds R + nt - 1 zeroed counters; a value out of
// range or seen twice records DEV_BAD_INDEX in the status word.
__global__ void check_perms(const uint32_t* slot, int R, const uint32_t* order, int m, unsigned* seen,
                            DevStatus* st) {
    for (int x = blockIdx.x * blockDim.x + threadIdx.x; x < R + m; x += gridDim.x * blockDim.x) {
        const bool is_slot = x < R;
        const uint32_t v = is_slot ? slot[x] : order[x - R];
        const uint32_t lim = is_slot ? (uint32_t)R : (uint32_t)m;
        bool bad = v >= lim;
        if (!bad) bad = atomicAdd(seen + (is_slot ? 0 : R) + v, 1u) != 0u;
        if (bad && atomicCAS(&st->error, 0, (int)DEV_BAD_INDEX) == 0) {
            st->where = is_slot ? 1 : 2;
            st->aux0 = is_slot ? x : x - R;
            st->aux1 = v;
        }
    }
}

// Every best energy starts at "none yet" (the largest int64, as elsewhere in
// the library).
__global__ void fill_no_best(long long* bestE, int R) {
    for (int x = blockIdx.x * blockDim.x + threadIdx.x; x < R; x += gridDim.x * blockDim.x) bestE[x] = kNoBest;
}

// Bump allocator over the scratch array (256-byte aligned regions).
struct Carve {
    size_t off = 0;
    size_t take(size_t bytes) {
        const size_t o = off;
        off = (off + bytes + 255) & ~size_t(255);
        return o;
    }
};

}  // namespace
}  // namespace pticm

using namespace pticm;

extern "C" int pticm_run_noalloc(const pticm_problem* p, const pticm_opts* o, const double* beta, uint32_t nt,
                                 int32_t nc, const pticm_noalloc_io* io, uint64_t step0, uint64_t pt_steps,
                                 void* stream) {
    if (!p || !o || !beta || !io || !io->spins_in || !io->spins_out || !io->energy_out)
        return noalloc_fail(PTICM_ERR_INVALID, "null argument");
    if (o->nt != nt || nt < 2) return noalloc_fail(PTICM_ERR_INVALID, "nt must match the options and be >= 2");
    if (o->chains < 1 || o->chains > 16 || (o->icm && (o->chains % 2)))
        return noalloc_fail(PTICM_ERR_INVALID, "chains must be in [1, 16] (even with ICM)");
    if (o->sweeps < 1 || o->exchange > 1 || o->icm_algo > 3) return noalloc_fail(PTICM_ERR_INVALID, "invalid options");
    for (uint32_t k = 0; k < nt; k++)
        if (!std::isfinite(beta[k])) return noalloc_fail(PTICM_ERR_INVALID, "non-finite inverse temperature");
    const HostProblem& P = problem_host(p);
    const int R = (int)(nt * o->chains);
    InstanceDesc D{};
    D.n = (int32_t)P.n;
    D.n_pad = (int32_t)((P.n + 15) & ~15ll);
    D.nnz = (int32_t)P.dadj.size();
    D.ncolors = P.ncolors;
    D.kmax = P.kmax;
    D.nt = (int32_t)nt;
    D.chains = (int32_t)o->chains;
    D.R = R;
    D.has_h = P.has_h ? 1 : 0;
    std::vector<uint32_t> thr;
    std::vector<double> ptab;
    D.nc = ladder_tables(P, beta, (int)nt, nc, o->icm != 0, (int)o->chains, thr, ptab);
    LaunchConfig cfg;
    std::string msg;
    if (int rc = choose_config(P, *o, false, D, cfg, msg)) return noalloc_fail(rc, msg);
    if (cfg.state_global || cfg.field_gather)
        return noalloc_fail(PTICM_ERR_UNSUPPORTED, "the replicas do not fit shared memory; use pticm_create/pticm_run");
    finish_desc(D, P, *o, cfg);

    // carve the scratch array
    const size_t n = (size_t)D.n, npad = (size_t)D.n_pad, nnz = (size_t)D.nnz, RR = (size_t)R;
    Carve cv;
    const size_t o_status = cv.take(sizeof(DevStatus)), o_abort = cv.take(sizeof(int)), o_bar = cv.take(2 * sizeof(unsigned));
    const size_t o_desc = cv.take(sizeof(InstanceDesc)), o_soff = cv.take(((size_t)cfg.group + 1) * 4),
                 o_sched = cv.take((size_t)cfg.group * 8), o_rinst = cv.take(RR * 4);
    const size_t o_row = cv.take((n + 5) * 4), o_adj = cv.take((nnz + 4) * 4), o_col = cv.take(((size_t)D.ncolors + 5) * 4);
    const size_t o_h = cv.take((n + 4) * 4), o_perm = cv.take((n + 4) * 4), o_beta = cv.take((size_t)nt * 8);
    const size_t o_thr = cv.take(thr.size() * 4 + 16);
    const size_t o_spins = cv.take(RR * npad), o_fields = cv.take(RR * npad * 4), o_E = cv.take(RR * 8);
    const size_t o_pub = cv.take(2 * RR * npad), o_Epub = cv.take(2 * RR * 8 * kPubStride);
    const size_t o_flips = cv.take(RR * 8), o_bestE = cv.take(RR * 8), o_bestS = cv.take(RR * 8);
    const size_t o_bstate = cv.take(RR * npad), o_slot = cv.take(RR * 4), o_order = cv.take((size_t)nt * 4);
    const size_t o_att = cv.take(RR * 8), o_succ = cv.take(RR * 8);
    const size_t o_seen = cv.take((RR + nt) * 4);
    if (cv.off > (size_t)PTICM_NOALLOC_SCRATCH_BYTES)
        return noalloc_fail(PTICM_ERR_UNSUPPORTED,
                            "run needs " + std::to_string(cv.off) + " bytes of working memory; pticm_run_noalloc is limited to " +
                                std::to_string((size_t)PTICM_NOALLOC_SCRATCH_BYTES) + " bytes (use pticm_create/pticm_run)");
    void* basev = nullptr;
    if (int rc = scratch_address(&basev)) return rc;
    unsigned char* base = static_cast<unsigned char*>(basev);
    cudaStream_t st = static_cast<cudaStream_t>(stream);

    // inputs of the engine layout: host-built tables copied into the array
    std::vector<int32_t> soff, sched, rinst(RR, 0), perm(P.perm);
    single_instance_schedule(cfg.group, soff, sched);
    std::vector<uint32_t> slot0(RR), order0(nt, 0);
    for (int r = 0; r < R; r++) slot0[r] = (uint32_t)r;
    for (uint32_t k = 0; k + 1 < nt; k++) order0[k] = k;
    NA_CK(cudaMemcpyAsync(base + o_desc, &D, sizeof(D), cudaMemcpyHostToDevice, st));
    NA_CK(cudaMemcpyAsync(base + o_soff, soff.data(), soff.size() * 4, cudaMemcpyHostToDevice, st));
    NA_CK(cudaMemcpyAsync(base + o_sched, sched.data(), sched.size() * 4, cudaMemcpyHostToDevice, st));
    NA_CK(cudaMemcpyAsync(base + o_rinst, rinst.data(), rinst.size() * 4, cudaMemcpyHostToDevice, st));
    NA_CK(cudaMemcpyAsync(base + o_row, P.drow.data(), P.drow.size() * 4, cudaMemcpyHostToDevice, st));
    if (nnz) NA_CK(cudaMemcpyAsync(base + o_adj, P.dadj.data(), nnz * 4, cudaMemcpyHostToDevice, st));
    NA_CK(cudaMemcpyAsync(base + o_col, P.color_off.data(), P.color_off.size() * 4, cudaMemcpyHostToDevice, st));
    NA_CK(cudaMemcpyAsync(base + o_h, P.dh.data(), n * 4, cudaMemcpyHostToDevice, st));
    NA_CK(cudaMemcpyAsync(base + o_perm, perm.data(), n * 4, cudaMemcpyHostToDevice, st));
    NA_CK(cudaMemcpyAsync(base + o_beta, beta, (size_t)nt * 8, cudaMemcpyHostToDevice, st));
    NA_CK(cudaMemcpyAsync(base + o_thr, thr.data(), thr.size() * 4, cudaMemcpyHostToDevice, st));
    // everything a run starts from zero
    NA_CK(cudaMemsetAsync(base + o_status, 0, sizeof(DevStatus), st));
    NA_CK(cudaMemsetAsync(base + o_abort, 0, sizeof(int), st));
    NA_CK(cudaMemsetAsync(base + o_bar, 0, 2 * sizeof(unsigned), st));
    NA_CK(cudaMemsetAsync(base + o_flips, 0, RR * 8, st));
    NA_CK(cudaMemsetAsync(base + o_bestS, 0, RR * 8, st));
    NA_CK(cudaMemsetAsync(base + o_att, 0, RR * 8, st));
    NA_CK(cudaMemsetAsync(base + o_succ, 0, RR * 8, st));
    if (io->slot_to_replica)
        NA_CK(cudaMemcpyAsync(base + o_slot, io->slot_to_replica, RR * 4, cudaMemcpyDeviceToDevice, st));
    else
        NA_CK(cudaMemcpyAsync(base + o_slot, slot0.data(), RR * 4, cudaMemcpyHostToDevice, st));
    if (io->pair_order)
        NA_CK(cudaMemcpyAsync(base + o_order, io->pair_order, (size_t)(nt - 1) * 4, cudaMemcpyDeviceToDevice, st));
    else
        NA_CK(cudaMemcpyAsync(base + o_order, order0.data(), (size_t)nt * 4, cudaMemcpyHostToDevice, st));
    // the slot map and pair order must be permutations before the engine
    // indexes with them (also those passed in by the caller)
    NA_CK(cudaMemsetAsync(base + o_seen, 0, (RR + nt) * 4, st));
    check_perms<<<std::max(1, std::min(64, (int)((RR + nt + 255) / 256))), 256, 0, st>>>(
        reinterpret_cast<const uint32_t*>(base + o_slot), R, reinterpret_cast<const uint32_t*>(base + o_order),
        (int)nt - 1, reinterpret_cast<unsigned*>(base + o_seen), reinterpret_cast<DevStatus*>(base + o_status));
    NA_CK(cudaGetLastError());
    {
        DevStatus cs{};
        NA_CK(cudaMemcpyAsync(&cs, base + o_status, sizeof(cs), cudaMemcpyDeviceToHost, st));
        NA_CK(cudaStreamSynchronize(st));
        if (cs.error)
            return noalloc_fail(PTICM_ERR_INVALID,
                                std::string(cs.where == 1 ? "slot_to_replica is not a permutation of 0..R-1"
                                                          : "pair_order is not a permutation of 0..nt-2") +
                                    " (entry " + std::to_string(cs.aux0) + " = " + std::to_string(cs.aux1) + ")");
    }
    fill_no_best<<<std::max(1, std::min(64, (R + 255) / 256)), 256, 0, st>>>(
        reinterpret_cast<long long*>(base + o_bestE), R);
    NA_CK(cudaGetLastError());

    EngineArgs A{};
    A.desc = reinterpret_cast<const InstanceDesc*>(base + o_desc);
    A.sched_off = reinterpret_cast<const int32_t*>(base + o_soff);
    A.sched = reinterpret_cast<const int32_t*>(base + o_sched);
    A.n_inst = 1;
    A.n_blocks = cfg.group;
    A.row = reinterpret_cast<const int32_t*>(base + o_row);
    A.adj = reinterpret_cast<const uint32_t*>(base + o_adj);
    A.col = reinterpret_cast<const int32_t*>(base + o_col);
    A.hpool = reinterpret_cast<const int32_t*>(base + o_h);
    A.beta = reinterpret_cast<const double*>(base + o_beta);
    A.thr = reinterpret_cast<const uint32_t*>(base + o_thr);
    A.ptab = nullptr;
    A.perm = nullptr;
    A.spins = reinterpret_cast<int8_t*>(base + o_spins);
    A.fields = reinterpret_cast<int32_t*>(base + o_fields);
    A.energy = reinterpret_cast<long long*>(base + o_E);
    A.spins_pub = reinterpret_cast<int8_t*>(base + o_pub);
    A.spins_pub_half = (long long)RR * npad;
    A.energy_pub = reinterpret_cast<long long*>(base + o_Epub);
    A.energy_pub_half = R;
    A.flips = reinterpret_cast<unsigned long long*>(base + o_flips);
    A.best_E = reinterpret_cast<long long*>(base + o_bestE);
    A.best_sweep = reinterpret_cast<unsigned long long*>(base + o_bestS);
    A.best_state = reinterpret_cast<int8_t*>(base + o_bstate);
    A.slot_rep = reinterpret_cast<uint32_t*>(base + o_slot);
    A.xorder = reinterpret_cast<uint32_t*>(base + o_order);
    A.xcursor = nullptr;
    A.attempts = reinterpret_cast<unsigned long long*>(base + o_att);
    A.successes = reinterpret_cast<unsigned long long*>(base + o_succ);
    A.bar = reinterpret_cast<unsigned int*>(base + o_bar);
    A.flag_barrier = energy_bound(P) < (1ll << 31) ? 1 : 0;   // every energy fits the word's 32 bits
    A.abort_flag = reinterpret_cast<int*>(base + o_abort);
    A.status = reinterpret_cast<DevStatus*>(base + o_status);
    A.sweeps = (int)o->sweeps;
    A.seed = o->seed;
    A.sm = cfg.plan;
    A.flags = engine_flags(P, *o);
    A.prof = nullptr;

    // initial spins -> engine layout, fields and energies from scratch
    const int32_t* d_perm = reinterpret_cast<const int32_t*>(base + o_perm);
    import_spins<<<std::max(1, std::min(1024, (int)((RR * npad + 255) / 256))), 256, 0, st>>>(
        io->spins_in, A.spins, d_perm, D.n, D.n_pad, R);
    NA_CK(cudaGetLastError());
    NA_CK(launch_recompute(A, reinterpret_cast<const int32_t*>(base + o_rinst), R, 1, nullptr, nullptr, nullptr, st));
    NA_CK(cudaMemcpyAsync(A.best_state, A.spins, RR * npad, cudaMemcpyDeviceToDevice, st));

    uint64_t left = pt_steps, step = step0;
    while (left > 0) {
        const int chunk = (int)std::min<uint64_t>(left, 1u << 16);
        A.step0 = step;
        A.nsteps = chunk;
        A.phase_mask = PHASE_SWEEP | PHASE_EXCHANGE | PHASE_ICM;
        NA_CK(cudaMemsetAsync(base + o_bar, 0, 2 * sizeof(unsigned), st));
        NA_CK(launch_engine(A, cfg.threads, false, cfg.block_team, cfg.narrow, cfg.group > 1, st));
        step += (uint64_t)chunk;
        left -= (uint64_t)chunk;
    }

    // outputs into the caller's buffers
    export_spins<<<std::max(1, std::min(1024, (int)((RR * n + 255) / 256))), 256, 0, st>>>(
        A.spins, io->spins_out, d_perm, D.n, D.n_pad, R);
    NA_CK(cudaGetLastError());
    NA_CK(cudaMemcpyAsync(io->energy_out, A.energy, RR * 8, cudaMemcpyDeviceToDevice, st));
    if (io->slot_to_replica)
        NA_CK(cudaMemcpyAsync(io->slot_to_replica, A.slot_rep, RR * 4, cudaMemcpyDeviceToDevice, st));
    if (io->pair_order)
        NA_CK(cudaMemcpyAsync(io->pair_order, A.xorder, (size_t)(nt - 1) * 4, cudaMemcpyDeviceToDevice, st));
    if (io->swap_attempts) NA_CK(cudaMemcpyAsync(io->swap_attempts, A.attempts, RR * 8, cudaMemcpyDeviceToDevice, st));
    if (io->swap_successes) NA_CK(cudaMemcpyAsync(io->swap_successes, A.successes, RR * 8, cudaMemcpyDeviceToDevice, st));
    if (io->best_energy_out) NA_CK(cudaMemcpyAsync(io->best_energy_out, A.best_E, RR * 8, cudaMemcpyDeviceToDevice, st));
    if (io->best_states_out) {
        export_spins<<<std::max(1, std::min(1024, (int)((RR * n + 255) / 256))), 256, 0, st>>>(
            A.best_state, io->best_states_out, d_perm, D.n, D.n_pad, R);
        NA_CK(cudaGetLastError());
    }
    DevStatus hs{};
    NA_CK(cudaMemcpyAsync(&hs, base + o_status, sizeof(hs), cudaMemcpyDeviceToHost, st));
    NA_CK(cudaStreamSynchronize(st));
    if (hs.error)
        return noalloc_fail(PTICM_ERR_DEVICE, "pticm_run_noalloc: device reported error " + std::to_string(hs.error) +
                                                  " at site " + std::to_string(hs.where));
    return PTICM_OK;
}
