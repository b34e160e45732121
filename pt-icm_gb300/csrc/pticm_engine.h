// pticm_engine.h -- layout contract between the host runtime and the PT-ICM
// engine kernel.  Plain structs, shared by host (.cc) and device (.cu) code.
#pragma once
#include <cstdint>

namespace pticm {

// First device-side failure of a launch (error 0 = none).
struct DevStatus {
    int error;
    int where;
    long long aux0;
    long long aux1;
};

// One PT instance (a graph and its 2..C replica chains) inside a launch.
// Sites are renumbered so that colour classes are contiguous: site i of the
// device layout is original site perm[i].  Every pool offset is in elements.
struct InstanceDesc {
    int32_t n;          // spins
    int32_t n_pad;      // row stride of per-replica arrays (multiple of 16)
    int32_t nnz;        // directed adjacency entries (2M for sparse inputs)
    int32_t ncolors;    // colour classes
    int32_t kmax;       // largest dE/2 = max_i (|h_i| + sum_j |J_ij|)
    int32_t nt;         // temperatures per chain
    int32_t chains;     // replicas per temperature
    int32_t R;          // replicas = nt * chains
    int32_t nc;         // ICM temperatures (coldest nc slots of each chain pair)
    int32_t has_h;      // linear terms present
    int32_t group;      // blocks that share this instance
    int32_t rpc;        // replicas per block (R = group * rpc)
    int32_t first_block;
    int32_t inst_id;    // stable id used in RNG counters (< 65536)
    int32_t icm_algo;   // ENGINE_ICM_* cluster search of this instance
    int32_t stage;      // 1: adjacency staged into shared memory by bulk copy
    int32_t teams;      // ICM warp teams of a block (scratch of icm_team_bytes(n_pad) each)
    int32_t pad0;
    int64_t row_off;    // int32 pool: n+1 row starts (relative to the instance)
    int64_t adj_off;    // uint32 pool: nnz packed entries (col << 8 | (uint8)J)
    int64_t col_off;    // int32 pool: ncolors+1 colour-class starts
    int64_t h_off;      // int32 pool: n linear terms
    int64_t beta_off;   // double pool: nt values
    int64_t thr_off;    // uint32 pool: nt*(kmax+1) acceptance thresholds
    int64_t ptab_off;   // double pool: nt*(kmax+1) exp(-beta*dE) (replay)
    int64_t rep_off;    // first replica of the instance in the replica pools
    int64_t spin_off;   // first byte of the instance in the spin pools
    int64_t perm_off;   // int32 pool: original site -> device site (replay)
    // optional energy histogram rows (R rows of hist_nbins bins at hist_off of
    // the launch's histogram pool; bin b holds E = hist_lo + 2b); 0 bins: none
    int64_t hist_off;
    int64_t hist_lo;
    int64_t hist_nbins;
};

// Shared-memory plan of a launch (bytes), identical for every block.
struct SmemPlan {
    uint32_t total;
    uint32_t mbar;
    uint32_t row, adj;          // staged adjacency (when stage_adj)
    uint32_t col, h;
    uint32_t spin, field;       // rpc * n_pad
    uint32_t thr;               // rpc * (kmax+1)
    uint32_t ptab;              // replay: nt * (kmax+1) doubles
    uint32_t slot, rslot, order, beta, dbeta;
    uint32_t E, dEp, flp, bestE, flips, improved;
    uint32_t att, succ;
    uint32_t xlogu, xrand, xlevel, xpos;
    uint32_t icm, icm_team_bytes;
    uint32_t mag;               // rpc magnetisations (observables)
    uint32_t misc;
    int32_t stage_adj;
    int32_t state_global;       // replica spins/fields and ICM scratch in device memory (large instances)
    int32_t field_gather;       // spins in shared memory, no stored fields: each visit gathers the local
                                // field from the neighbours' spins; ICM scratch and thresholds in device memory
    int32_t teams;              // ICM teams (warps, or one block-wide team)
    int32_t max_n_pad, max_kmax, max_R, max_nt;
    int32_t icm_split;          // field_gather with several replicas: the block team's ICM scratch in shared
                                // memory (at icm), its overlap list in device memory
};

// Trace of every random decision of the reference's sequential algorithm,
// consumed by the replay variant of the kernel.
struct ReplayArgs {
    const double* uniforms;         // sweep uniforms, (step, sweep, replica) order
    const uint64_t* sweep_offsets;  // pts*sweeps*R + 1
    const int32_t* xchg_slot;       // pts * chains*(nt-1)
    const double* xchg_logu;
    const int64_t* icm_seed;        // pts * nc (original site or -1)
    uint64_t n_uniforms, n_xchg, n_icm;
};

struct EngineArgs {
    const InstanceDesc* desc;
    // schedule: block b runs jobs sched_off[b] .. sched_off[b+1]-1 in order;
    // job j is instance sched[2j] as rank sched[2j+1] of its group.  Every
    // block lists its jobs in one global order, so the blocks of a group
    // meet at the group barrier (all blocks are co-resident).
    const int32_t* sched_off;
    const int32_t* sched;
    int32_t n_inst;
    int32_t n_blocks;
    // graph pools
    const int32_t* row;
    const uint32_t* adj;
    const int32_t* col;
    const int32_t* hpool;
    const double* beta;
    const uint32_t* thr;
    const double* ptab;
    const int32_t* perm;
    // replica pools
    int8_t* spins;                // master copy
    int32_t* fields;
    long long* energy;
    int8_t* spins_pub;            // 2 halves, parity of the PT step
    long long spins_pub_half;     // elements per half
    long long* energy_pub;        // 2 * total replicas (x kPubStride words with flag_barrier)
    long long energy_pub_half;
    unsigned long long* flips;
    long long* best_E;
    unsigned long long* best_sweep;
    int8_t* best_state;
    // per-instance PT bookkeeping (instance-local replica ids, slot = chain*nt + k)
    uint32_t* slot_rep;           // total replicas
    uint32_t* xorder;             // per instance nt entries (at rep_off)
    uint32_t* xcursor;            // per instance
    unsigned long long* attempts; // per slot
    unsigned long long* successes;
    unsigned int* bar;            // 2 words per instance
    int* abort_flag;
    DevStatus* status;
    // run control
    unsigned long long step0;
    int32_t nsteps;
    int32_t sweeps;
    int32_t phase_mask;           // 1 sweep, 2 exchange, 4 ICM
    int32_t flags;                // ENGINE_* flags
    unsigned long long seed;
    unsigned long long* prof;     // optional: per block, clock64 cycles per phase (PROF_PHASES)
    unsigned long long* job_ns;   // optional: per job, ns from the start of its step 1 to its end
    uint8_t* icm_pool;            // state_global: per block ICM scratch (icm_pool_stride bytes)
    long long icm_pool_stride;
    // optional per-slot energy histograms (the pilot run of the multihistogram
    // ladder): after the sweeps of every step >= hist_from, slot k of an
    // instance counts the energy E of its replica in bin (E - hist_lo) / 2 of
    // its row k (InstanceDesc::hist_*)
    unsigned int* hist;
    unsigned long long hist_from;
    // optional magnetisation observables (with the histograms): per slot
    // sum of M = sum_i s_i and of M^2 at obs[2 (rep_off + slot)], and the
    // published M of every replica (two parity halves, like energy_pub)
    long long* obs;
    long long* mag_pub;
    SmemPlan sm;
    ReplayArgs replay;
    // optional ICM controls: per pair q a seed site in the original numbering
    // (-1: the random choice, -2: skip the pair); icm_exact flips the seed's
    // cluster itself, never the rest of the overlap
    const long long* icm_force;
    int32_t icm_exact;
    // bounded waits: the limit of every wait on other blocks or on bulk
    // copies (0: kWaitLimitNs), and arrivals a group barrier counts beyond
    // the group's blocks (0 in production; a test hook that makes the
    // barrier's wait run out)
    int32_t bar_phantom;
    unsigned long long wait_limit_ns;
    // The per-step exchange of a group's energies: 1 = tagged energy words
    // (energy_pub holds tag << 32 | energy; every energy of the problem fits
    // 32 bits), 0 = the counting group barrier, then plain energy loads.
    // pub_base + (step within the launch) is the tag; launch_engine sets it.
    int32_t flag_barrier;
    uint32_t pub_base;
};

enum EngineFlags : int32_t {
    ENGINE_BEST_PER_PHASE = 1,    // track the best state after every colour phase
    ENGINE_REPLAY = 2,            // sequential sweep + traced decisions
    ENGINE_EXCHANGE_EVEN_ODD = 4, // deterministic even/odd exchange rounds
    // cluster algorithm of the ICM phase (bits 3-4)
    ENGINE_ICM_BFS = 0,
    ENGINE_ICM_UNION_FIND = 8,
    ENGINE_ICM_LABEL_PROP = 16,
    ENGINE_ICM_MASK = 24,
};

// Shared-memory scratch of one ICM team for an instance of n_pad sites: BFS
// queue / labels (4 B per site), overlap flags (1 B per site), visited bits.
// Threads of a block of several replicas, or of a block team launched with
// the narrow bound (120 registers a thread).
constexpr int kNarrowThreads = 512;
// Published energy words (flag_barrier) sit one per 128-byte line, so that
// the blocks polling a group's words do not all queue on a few lines:
// energy_pub holds 2 * replicas * kPubStride words.
constexpr int kPubStride = 16;

inline constexpr uint32_t icm_team_bytes(int32_t n_pad) {
    return (uint32_t)((((uint64_t)n_pad * 5 + 4 * (((uint64_t)n_pad + 31) / 32)) + 15) & ~15ull);
}

// ICM scratch of a block: `teams` warp teams of icm_team_bytes each, or one
// block-wide team, which also lists the overlap sites (n_pad ints after its
// team scratch).
inline constexpr uint64_t icm_block_bytes(int32_t teams, int32_t n_pad) {
    return teams == 1 ? (uint64_t)icm_team_bytes(n_pad) + 4ull * (uint64_t)n_pad
                      : (uint64_t)teams * icm_team_bytes(n_pad);
}

enum PhaseBits : int32_t { PHASE_SWEEP = 1, PHASE_EXCHANGE = 2, PHASE_ICM = 4 };

// Phase timers: cycles spent per block in sweep, publish+barrier, exchange
// and ICM, plus the whole launch.
// Slots 5.. split ICM (overlap+count, seed choice, union, flip, energies) and
// the exchange (draws, dependency levels, attempts, reshuffle) as seen by
// thread 0 of the block; slots 14-20 split the union-find labelling of a
// block team (the two link rounds and the compression between them, the
// vote for the giant component, the pass that lists the sites outside it,
// their unions, and the cluster size), slot 21 is the sweep time of blocks
// whose replica takes part in an ICM pair of the step, and slot 22 counts
// the ICM pairs with a nonempty overlap (a count, not cycles).
enum ProfSlots : int32_t {
    PROF_SWEEP = 0, PROF_BARRIER = 1, PROF_EXCHANGE = 2, PROF_ICM = 3, PROF_TOTAL = 4,
    PROF_ICM_DIFF = 5, PROF_ICM_SEED = 6, PROF_ICM_UNION = 7, PROF_ICM_FLIP = 8, PROF_ICM_ENERGY = 9,
    PROF_X_DRAW = 10, PROF_X_LEVELS = 11, PROF_X_APPLY = 12, PROF_X_SHUFFLE = 13,
    PROF_UF_LINK0 = 14, PROF_UF_COMPRESS = 15, PROF_UF_LINK1 = 16, PROF_UF_VOTE = 17, PROF_UF_OUTSIDE = 18,
    PROF_UF_SUNION = 19, PROF_UF_SIZE = 20, PROF_SWEEP_ICM = 21, PROF_ICM_COUNT = 22,
    PROF_PHASES = 23
};

}  // namespace pticm
