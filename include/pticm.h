/*
 * pticm.h -- C ABI of the GB300 (sm_103a) PT-ICM engine.
 *
 * Parallel tempering with isoenergetic cluster moves for Ising spin glasses
 * and MaxCut on Gset graphs.  Every replica of a run is resident on one GPU;
 * one persistent kernel performs, per PT step, colour-class Metropolis
 * sweeps, replica exchange as a permutation of temperature slots, and
 * union-find cluster moves.
 *
 * Conventions: every function returns a pticm_status (0 = success); no
 * exceptions cross this boundary; pticm_last_error() describes the last
 * failure of the calling thread.  Buffers passed in are plain host memory and
 * are copied.  Spin states at this boundary are one byte per site, 0 or 1 in
 * the reference's bool convention (true = +1), in the ORIGINAL site order of
 * the problem file.  Energies follow the reference's sign convention
 * E = sum_i h_i s_i + sum_{i<j} J_ij s_i s_j.
 *
 * Each declaration cites the reference interface it replaces
 * (mxburns2022/PT-ICM, paths relative to that project).
 */
#ifndef PTICM_H
#define PTICM_H

#include <stddef.h>
#include <stdint.h>

/* The library is built with hidden visibility; only this C ABI is exported. */
#if defined(__GNUC__)
#define PTICM_API __attribute__((visibility("default")))
#else
#define PTICM_API
#endif

#ifdef __cplusplus
extern "C" {
#endif

typedef enum pticm_status {
    PTICM_OK = 0,
    PTICM_ERR_INVALID = 1,      /* bad argument or call order                  */
    PTICM_ERR_IO = 2,           /* unreadable or malformed problem file        */
    PTICM_ERR_UNSUPPORTED = 3,  /* e.g. non-integer couplings, self loops      */
    PTICM_ERR_CUDA = 4,         /* CUDA runtime failure                        */
    PTICM_ERR_DEVICE = 5,       /* a kernel reported a failure (bounded wait,  */
                                /* replay mismatch, bounds check)              */
    PTICM_ERR_NOMEM = 6,        /* host or device allocation failed            */
    PTICM_ERR_NODEVICE = 7      /* no CUDA device (the engine has no CPU path) */
} pticm_status;

typedef struct pticm_problem pticm_problem;
typedef struct pticm_ctx pticm_ctx;

/* ------------------------------------------------------------ problems -- */
typedef struct pticm_problem_info {
    int64_t n;              /* spins                                          */
    int64_t m;              /* edges as counted in the file header            */
    int64_t nnz;            /* directed adjacency entries                     */
    int32_t sparse;         /* reference's sparse/dense choice (density<10%)  */
    int32_t ncolors;        /* colour classes of the sweep order              */
    int32_t kmax;           /* largest |dE|/2                                 */
    int32_t has_linear;     /* nonzero linear terms                           */
    double char_scale;      /* max(mean w, var w): ICM temperature cutoff     */
    double total_weight;    /* sum of edge weights (cut = (W - E_J)/2)        */
} pticm_problem_info;

/* Problem(path, seed, burn_in)  src/problem.cc:183-247.  Honours the
 * reference's rules: ".gset"/".ising" anywhere in the path means 0-based
 * vertices, else 1-based; a missing weight is 1; ".ising" files carry a
 * linear-term block.  Couplings and linear terms must be integers in
 * [-127, 127] (PTICM_ERR_UNSUPPORTED otherwise). */
PTICM_API int pticm_problem_load_gset(const char* path, pticm_problem** out);

/* Problem(weights, src, dest, linear, seed, burn_in, N, M)
 * include/problem.hh:43-62.  `h` may be NULL. */
PTICM_API int pticm_problem_from_coo(int64_t n, int64_t m, const int32_t* src, const int32_t* dst,
                           const double* w, const double* h, pticm_problem** out);

/* Problem(formulation, linear, seed, burn_in, N)  include/problem.hh:23-42:
 * a dense row-major n*n coupling matrix (only j != i entries are used; zero
 * entries are not edges).  `h` may be NULL. */
PTICM_API int pticm_problem_from_dense(int64_t n, const double* J, const double* h, pticm_problem** out);

PTICM_API void pticm_problem_free(pticm_problem* p);
PTICM_API int pticm_problem_get_info(const pticm_problem* p, pticm_problem_info* out);

/* The sweep's colour class of every site (original numbering), n entries.
 * The engine updates a class in parallel, so no edge may join two sites of
 * one class; the classes come from a two-colouring of bipartite graphs, else
 * the better of Welsh-Powell and DSatur.  Host only (no device work). */
PTICM_API int pticm_problem_get_colouring(const pticm_problem* p, int32_t* colour);

/* Problem::energy, Problem::maxcut, Problem::calculate_dE
 * src/problem.cc:33-162, computed on the GPU for `count` states
 * (count*n bytes).  `dE` (count*n doubles) may be NULL. */
PTICM_API int pticm_problem_evaluate(const pticm_problem* p, int64_t count, const uint8_t* states,
                           double* energy, double* maxcut, double* dE);

/* --------------------------------------------------------- PT contexts -- */
typedef struct pticm_opts {
    uint64_t seed;          /* -s                                             */
    uint32_t nt;            /* -r: temperatures per chain                     */
    uint32_t chains;        /* replicas per temperature (2 in the reference)  */
    uint32_t sweeps;        /* --sweeps per PT step                           */
    uint32_t icm;           /* --icm                                          */
    uint32_t exchange;      /* 1 even/odd rounds (default), 0 the reference's */
                            /* shuffled attempt order (src/replica_exchange.cc)*/
    uint32_t best_per_phase;/* 1: best state checked after every colour class,*/
                            /* 0 (default): after every sweep                 */
    uint32_t block_threads; /* 0 = automatic                                  */
    uint32_t replicas_per_block; /* 0 = automatic                             */
    uint32_t icm_algo;      /* cluster search: 0 auto, 1 breadth-first,       */
                            /* 2 union-find, 3 label propagation              */
} pticm_opts;

PTICM_API void pticm_opts_default(pticm_opts* o);

/* State of solve() between initialisation and reporting
 * (src/solver.cc:16-166, include/mpi_defs.hh:33-65): all replicas of the
 * problem resident on the current CUDA device. */
PTICM_API int pticm_create(const pticm_problem* p, const pticm_opts* o, pticm_ctx** out);
PTICM_API void pticm_destroy(pticm_ctx* c);

/* initialize_temperatures (src/initialization.cc:103-191) with an explicit
 * ladder of nt inverse temperatures (slot k of every chain gets beta[k]).
 * The ICM pair count follows src/initialization.cc:158-164 (entries from the
 * top slot down while beta >= char_scale) unless `nc` >= 0 sets it. */
PTICM_API int pticm_set_ladder(pticm_ctx* c, const double* beta, uint32_t nt, int32_t nc);

/* beta_linspace (src/utils.cc:6-22), linear in beta, same FP64 steps. */
PTICM_API int pticm_beta_linspace(double* beta, double T0, double T1, uint64_t nt, int inverse);

/* initialize_replicas (src/initialization.cc:63-76): Bernoulli(1/2) spins
 * from a counter-based stream, then a from-scratch field/energy pass. */
PTICM_API int pticm_init_states(pticm_ctx* c, uint64_t seed);
/* Explicit initial spins: R*n bytes (0/1), replica r = chain*nt + k. */
PTICM_API int pticm_set_states(pticm_ctx* c, const uint8_t* states);

#define PTICM_PHASE_SWEEP 1u
#define PTICM_PHASE_EXCHANGE 2u
#define PTICM_PHASE_ICM 4u
#define PTICM_PHASE_ALL 7u

/* The PT loop (src/solver.cc:67-127): `pt_steps` steps of sweeps, exchange
 * and ICM. `phase_mask` selects phases (1 sweep, 2 exchange, 4 ICM; 7 = all)
 * so that each phase can be checked on its own. */
PTICM_API int pticm_run(pticm_ctx* c, uint64_t pt_steps, uint32_t phase_mask);

typedef struct pticm_stats {
    uint64_t pt_steps;      /* steps run so far                               */
    uint64_t attempts;      /* spin-flip attempts (every visited site)        */
    uint64_t flips;         /* accepted flips (num_of_flips, untruncated)     */
    uint64_t swaps;         /* accepted exchanges (num_of_swaps)              */
    uint32_t nt, chains, nc, replicas;
    double last_run_ms;     /* device time of the last pticm_run (CUDA events)*/
} pticm_stats;

/* swap_attempts / swap_successes per slot (2*nt entries for two chains, as
 * printed by src/solver.cc:152-153); either array may be NULL. */
PTICM_API int pticm_get_stats(pticm_ctx* c, pticm_stats* s, uint64_t* swap_attempts, uint64_t* swap_successes);

/* gather_best_energy_values (src/mpi_utils.cc:103-163): lowest energy seen
 * by any replica, the replica's sweep counter then, and that state (n bytes). */
PTICM_API int pticm_get_best(pticm_ctx* c, double* energy, uint64_t* sweep, uint8_t* state, int64_t* replica);

/* Current replicas: states (R*n bytes), energies (R), local fields
 * f_i = sum_j J_ij s_j (R*n, original site order) and the temperature slot
 * of each replica.  Any pointer may be NULL. */
PTICM_API int pticm_get_replicas(pticm_ctx* c, uint8_t* states, int64_t* energy, int32_t* fields, uint32_t* slot_of_replica);

/* Checkpoint of the PT state of a context: replicas, fields, energies, the
 * ladder, the slot map, the exchange order and cursor, best states, the
 * flip and swap counters, the step count (which keys every random stream)
 * and, when enabled, the energy histograms.  A context created from the same
 * problem with the same options and loaded from it continues bit for bit as
 * the uninterrupted run.  The reference has no checkpointing (a run is one
 * process from src/main.cc to the report). */
PTICM_API int pticm_checkpoint_save(pticm_ctx* c, const char* path);
PTICM_API int pticm_checkpoint_load(pticm_ctx* c, const char* path);

/* One ICM phase on the current states with caller-chosen seeds: icm(w, k)
 * (src/icm.cc:74-215) for every pair q = (c/2)*nc + (nt-1-k) of chains c,
 * c+1 at temperature slot k, on the same kernel and block layout as
 * pticm_run.  seeds[q] (count = nc * chains/2 entries) is the seed site in
 * the original numbering -- the reference's xor_icm draw (src/icm.cc:33),
 * which must lie where the pair differs after its global-flip rule
 * (src/icm.cc:20-28) -- or -1 for the engine's own draw, or -2 to leave the
 * pair alone.  exact = 1 flips the seed's cluster itself, as bfs_icm
 * (src/icm.cc:37-72) does; exact = 0 flips the smaller of the cluster and the
 * rest of the overlap, as production does (the two chains then hold each
 * other's result).  Counts as one PT step of the random streams. */
PTICM_API int pticm_icm_pairs(pticm_ctx* c, const int64_t* seeds, uint32_t count, int exact);

/* The exchange order of the reference-order exchange (exchange = 0): the nt-1
 * pair indices in the order the next attempts take them (chain_1_exchange_
 * order of src/initialization.cc:77-100 and src/replica_exchange.cc:86-91). */
PTICM_API int pticm_get_exchange_order(pticm_ctx* c, uint32_t* order);

/* Bounded waits.  Every wait of a kernel on other blocks (the group barrier
 * of a PT step) or on bulk copies gives up after limit_ns (0: the default,
 * 2 s), records where, and the call returns PTICM_ERR_DEVICE; the context
 * stays usable.  phantom_arrivals = 1 is a test hook: every group barrier
 * then waits for one member more than it has (a block, or a replica's
 * energy word, that never arrives), so each of its waits runs out
 * (the reference has no failure detection: src/initialization.cc:120-126 and
 * src/mpi_utils.cc:223-225 assert or exit). */
PTICM_API int pticm_set_wait_limit(pticm_ctx* c, uint64_t limit_ns, uint32_t phantom_arrivals);

/* The engine layout a context runs (chosen at pticm_init_states /
 * pticm_set_states): replicas per block, blocks, threads per block, ICM teams
 * per block (1: the whole block is one team), whether one block holds one
 * replica (block team) on the narrow-bound kernel, whether the adjacency is
 * staged into shared memory, and where the replicas live (0 shared memory,
 * 1 spins in shared memory with fields gathered at each visit, 2 device
 * memory).  No counterpart in the reference (one replica per MPI rank). */
typedef struct pticm_layout {
    uint32_t replicas_per_block, blocks, threads, icm_teams;
    int32_t block_team, narrow, adjacency_staged, state_mode;
} pticm_layout;
PTICM_API int pticm_get_layout(pticm_ctx* c, pticm_layout* out);

/* Ladder and slot -> replica map (beta_indices of src/replica_exchange.cc). */
PTICM_API int pticm_get_ladder(pticm_ctx* c, double* beta, uint32_t* slot_to_replica, uint32_t* nc);

/* From-scratch recompute of every replica's fields and energy on the GPU,
 * compared with the incrementally tracked values; `mismatches` counts
 * differing sites and energies (0 = bit-exact). */
PTICM_API int pticm_verify(pticm_ctx* c, uint64_t* mismatches);

/* Phase timers (tracing): when enabled, every block of the following
 * pticm_run calls accumulates clock64 cycles spent in the sweep, the
 * publish+barrier, the exchange and the ICM phases, and the whole launch,
 * then ICM split into overlap, seed choice, union, flip and energies, the
 * exchange split into draws, dependency levels, attempts and reshuffle, the
 * union-find labelling of a block-wide ICM team split into its first link
 * round, compression, second link round, giant-component vote, the pass
 * listing the sites outside the giant component, their unions and the
 * cluster size, and the sweep time of blocks whose replica is in an ICM pair
 * of the step (PTICM_PROFILE_SLOTS values).  pticm_get_profile converts them
 * to milliseconds at the device's maximum SM clock and reports the mean and
 * the maximum over blocks -- except the last slot, the number of ICM pairs
 * with a nonempty overlap a block ran; enabling again clears the counters. */
#define PTICM_PROFILE_SLOTS 23
PTICM_API int pticm_set_profiling(pticm_ctx* c, int enable);
PTICM_API int pticm_get_profile(pticm_ctx* c, double* mean_ms, double* max_ms);

/* Per-temperature energy histograms (the observables the reference's --log
 * path was to log, src/main.cc:490-530, and the multihistogram input): from PT
 * step `from_step` on, every step adds the energy of the replica at each slot
 * after its sweeps, in exact levels E = e_lo + 2*bin (every energy has the
 * parity of e_lo).  Enabling clears the counts. */
PTICM_API int pticm_enable_energy_histograms(pticm_ctx* c, uint64_t from_step);
/* Rows of slot k at hist[k*nbins ...] (R rows); pass hist = NULL to query
 * nbins and e_lo first. */
PTICM_API int pticm_get_energy_histograms(pticm_ctx* c, uint32_t* hist, int64_t* e_lo, uint64_t* nbins);

/* The observables of the reference's --log (src/main.cc:490-530, there
 * commented out) from the samples collected since pticm_enable_energy_
 * histograms' from_step, per temperature j < nt (chains merged): T = 1/beta,
 * C = beta^2 Var(E) / N, X = beta Var(M) / N, u = <E>/N, m = <M>/N with
 * M = sum_i s_i; samples = sample count.  Any output may be NULL. */
PTICM_API int pticm_get_observables(pticm_ctx* c, double* T, double* C, double* X, double* u, double* m,
                                    uint64_t* samples);

/* -------------------------------------------- multihistogram ladder -- */
/* get_beta (src/cae_estimator.cc:295-428) on the GPU: a pilot PT run
 * (gather_samples, :76-151: one chain of nt temperatures linear in beta from
 * max(beta(T0), beta(T1)) down, burn_in + samples steps, shuffled-order
 * exchange, no ICM) with per-temperature energy histograms accumulated in the
 * kernel, the FP64 multihistogram density of states (:155-253) on the GPU,
 * and the greedy constant-acceptance walk to pair acceptance r (:367-425).
 * beta_out (>= nt entries) receives the descending ladder, *count its length.
 * The reference calls it with estep 2 and r 0.4 (src/initialization.cc:110)
 * and a burn-in of 5000 (src/cae_estimator.cc:74). */
PTICM_API int pticm_cae_ladder(const pticm_problem* p, uint64_t seed, double T0, double T1, int inverse, uint32_t nt,
                     double estep, double step_size, double r, uint64_t samples, uint64_t burn_in,
                     double* beta_out, uint32_t* count);

/* The multihistogram fixed point alone (get_partition_iterate,
 * src/cae_estimator.cc:228-253) for caller histograms in make_histogram's
 * layout (:45-69): row j has hist_len[j] counts at hist_off[j], bin 0 at
 * energy emin[j], bin width estep; n samples per row.  Writes
 * nbins = ceil((max_emax - min_j emin[j]) / estep) values of ln g (up to
 * logdos_cap) and the nt values of ln Z; iterates until
 * sum_j ((lnZ_j - lnZ'_j) / lnZ'_j)^2 <= 1e-7. */
PTICM_API int pticm_mhist_dos(const uint32_t* hist, const uint64_t* hist_off, const uint64_t* hist_len, uint32_t nt,
                    const double* beta_hist, const double* emin, double estep, uint64_t n, double max_emax,
                    double* logdos, uint64_t logdos_cap, double* logZ, uint64_t* nbins, uint64_t* iterations);

/* The constant-acceptance walk alone (src/cae_estimator.cc:367-425) from a
 * density of states; host code (no GPU needed), O(nbins) per candidate. */
PTICM_API int pticm_cae_walk(const double* logdos, uint64_t nbins, double min_emin, double estep, double beta_start,
                   double beta_end, double step_size, double r, uint32_t num_temps, double* beta_out,
                   uint32_t* count);

/* --------------------------------------------------------------- replay -- */
/* The reference's sequential algorithm driven by a recorded trace of its
 * random decisions: per PT step, per sweep, per replica the uniforms
 * Replica::sweep consumed (src/replica.cc:31-38), the exchange pair slots
 * and log-uniforms (src/replica_exchange.cc:11-28), and the ICM seed sites
 * (src/icm.cc:33).  The context must have chains == 2 and a ladder of
 * distinct temperatures; its states are set with pticm_set_states. */
typedef struct pticm_trace {
    uint64_t pt_steps;
    const double* uniforms;        /* all sweep uniforms, concatenated          */
    uint64_t n_uniforms;
    const uint64_t* sweep_offsets; /* pt_steps*sweeps*R + 1 offsets             */
    const int32_t* xchg_slot;      /* pt_steps*2*(nt-1) slots                   */
    const double* xchg_logu;
    const int64_t* icm_seed;       /* pt_steps*nc seeds, original index or -1   */
} pticm_trace;

PTICM_API int pticm_replay(pticm_ctx* c, const pticm_trace* t);

/* ------------------------------------------------------ single replicas -- */
/* One replica in device memory, for code written in the reference's
 * per-replica shape (its solve loop, src/solver.cc:67-127, and get_beta's
 * pilot loop, src/cae_estimator.cc:112-140): int8 spins and int32 local
 * fields, the energy, the best energy and state, flip and sweep counters,
 * and the FP64 table exp(-beta dE) of its temperature (built on the host
 * with the reference's expression).  The bulk path (pticm_run) keeps its
 * replicas in a context instead. */
typedef struct pticm_replica pticm_replica;
typedef struct pticm_replica_info {
    double energy, beta, best_energy;   /* best_energy: DBL_MAX before the first accepted flip */
    uint64_t best_sweep, flips, sweeps;
} pticm_replica_info;

/* Replica(Problem&, beta, init_state, init_dE, energy) include/replica.hh:27-33,
 * src/replica.cc:40-60: n bytes of 0/1 spins; the local fields and the energy
 * are computed from them (calculate_dE); best energy "none yet". */
PTICM_API int pticm_replica_create(const pticm_problem* p, double beta, const uint8_t* state, pticm_replica** out);
/* Replica::operator= (include/replica.hh:54-67): a new replica with the same
 * spins, fields, energies, counters and temperature. */
PTICM_API int pticm_replica_copy(const pticm_replica* src, pticm_replica** out);
PTICM_API void pticm_replica_destroy(pticm_replica* r);
/* Replica::set_beta (include/replica.hh:44). */
PTICM_API int pticm_replica_set_beta(pticm_replica* r, double beta);
/* Replica::set_state with the fields and energy recomputed from it. */
PTICM_API int pticm_replica_set_state(pticm_replica* r, const uint8_t* state);
/* Replica::set_energy / set_ene (include/replica.hh:36,43): an integer energy. */
PTICM_API int pticm_replica_set_energy(pticm_replica* r, double energy);
/* Replica(..., log_ene, burn_in): log the energy after every site visit of
 * the sweeps after the first burn_in (src/replica.cc:10-12). */
PTICM_API int pticm_replica_set_logging(pticm_replica* r, int log_energy, uint64_t burn_in);
/* Replica::sweep (src/replica.cc:5-38) on the GPU: sites 0..n-1 in order, a
 * move with dE <= 0 accepted, else accepted iff the next uniform is below
 * exp(-beta dE); fields, energy, flips and best state as mh_accept.  The
 * uniforms are the caller's (Problem::rand_double draws, src/replica.cc:36);
 * pass n_uniforms >= the sites (one per site at most); *consumed receives how
 * many the sweep used, so that the caller's generator can be advanced by
 * exactly that many.  *energy (may be NULL) receives the energy after the
 * sweep; energy_log (n values, may be NULL) the energy after every site when
 * logging is on and the sweep is past the burn-in. */
PTICM_API int pticm_replica_sweep(pticm_replica* r, const double* uniforms, uint64_t n_uniforms, uint64_t* consumed,
                                  double* energy, double* energy_log);
/* Replica's getters (include/replica.hh:35-50): info, the state (n bytes),
 * dE_i = -2 s_i (h_i + f_i) (n doubles) and the best state; any may be NULL. */
PTICM_API int pticm_replica_get(pticm_replica* r, pticm_replica_info* info, uint8_t* state, double* dE,
                                uint8_t* best_state);

/* xor_icm (src/icm.cc:8-35) on two states of n 0/1 bytes, without its seed
 * draw, on the GPU: s1 is negated when more than n/2 sites differ; *count
 * receives the number of differing sites and `sites` (n entries, may be
 * NULL) their indices ascending -- the population std::sample draws the seed
 * from (src/icm.cc:33). */
PTICM_API int pticm_problem_icm_overlap(const pticm_problem* p, uint8_t* s1, const uint8_t* s2, uint64_t* count,
                                        int64_t* sites);
/* bfs_icm (src/icm.cc:37-72) on the GPU: the seed's connected set of sites
 * where s1 and s2 differ is flipped in both. */
PTICM_API int pticm_problem_icm_cluster(const pticm_problem* p, int64_t seed, uint8_t* s1, uint8_t* s2);
/* Problem::incremental_dE (src/problem.cc:164-181) on the GPU: dE (n
 * doubles) after site `index` of `state` (its value before the flip) flips. */
PTICM_API int pticm_problem_incremental_dE(const pticm_problem* p, double* dE, const uint8_t* state,
                                           uint32_t index);

/* ----------------------------------------------- no device allocation -- */
/* For callers that cannot call cudaMalloc (their host framework owns every
 * device allocation and hands out buffers, or they must avoid the implicit
 * synchronisation of cudaMalloc/cudaFree): a complete PT run of `pt_steps`
 * steps (sweeps, exchange, ICM, as pticm_run) whose working memory lives in a
 * fixed device array of PTICM_NOALLOC_SCRATCH_BYTES inside this library.
 * This entry point has no counterpart in the reference.
 *
 * The caller passes device buffers for inputs and outputs (below); the run
 * starts from `spins_in` (fields and energies are recomputed from them) and
 * uses the steps step0..step0+pt_steps-1 of the counter-based random streams,
 * so chaining calls with step0 advanced continues one trajectory.  It calls
 * no cudaMalloc, cudaFree or allocating library routine.  Runs whose working
 * set exceeds the array (about 11 bytes per replica-site plus the graph) are
 * rejected with PTICM_ERR_UNSUPPORTED.  The first call on a device resolves
 * the array's address (make it before any stream capture); every GPU that
 * loads the library holds the array until exit; all calls share it, so calls
 * that overlap on the GPU race. `stream` is a cudaStream_t (NULL = legacy
 * default stream); the call returns after the stream has finished the run. */
#define PTICM_NOALLOC_SCRATCH_BYTES (8u << 20)

typedef struct pticm_noalloc_io {
    const uint8_t* spins_in;     /* device, R*n bytes (0/1, original site order), */
                                 /* replica r = chain*nt + k                     */
    uint8_t* spins_out;          /* device, R*n bytes; may be spins_in           */
    int64_t* energy_out;         /* device, R energies                           */
    uint32_t* slot_to_replica;   /* device, R, in/out; NULL: identity start       */
    uint32_t* pair_order;        /* device, nt-1, in/out (reference exchange     */
                                 /* order); NULL: ascending start                */
    uint64_t* swap_attempts;     /* device, R: this call's counts, or NULL        */
    uint64_t* swap_successes;    /* device, R, or NULL                           */
    int64_t* best_energy_out;    /* device, R: lowest energy seen this call, or NULL */
    uint8_t* best_states_out;    /* device, R*n: the matching states, or NULL    */
} pticm_noalloc_io;

PTICM_API int pticm_run_noalloc(const pticm_problem* p, const pticm_opts* o, const double* beta, uint32_t nt, int32_t nc,
                      const pticm_noalloc_io* io, uint64_t step0, uint64_t pt_steps, void* stream);

/* --------------------------------------------------- tensor-core GEMM -- */
/* A[M x K] . B[N x K]^T + bias on the tcgen05 tensor cores (BF16 operands
 * given as raw uint16 bit patterns, K-major; FP32 accumulation; K a multiple
 * of 64), with the epilogue of the surrogate network's layers: C receives the
 * FP32 result before the activation, C_bf16 (may be NULL) the BF16 output
 * after it (act 0 = none, 1 = SiLU), as the hidden layers store it.  Host
 * buffers; used to check the network's GEMM against a reference. */
PTICM_API int pticm_tc_gemm_check(int M, int N, int K, const uint16_t* A, const uint16_t* B, const float* bias,
                                  int act, float* C, uint16_t* C_bf16);
/* Device time of the tensor-core GEMM at M x N x K (bf16 operands and
 * output, FP32 accumulation), averaged over `iters` back-to-back launches
 * after one warm-up; tflops = 2 M N K / time. */
PTICM_API int pticm_tc_gemm_bench(int M, int N, int K, int iters, double* ms_per_gemm, double* tflops);

/* ------------------------------------------------------------ batching -- */
/* Many instances (problems of any sizes, same nt and chains) in one
 * persistent cooperative launch: instance i is split over g_i co-resident
 * blocks that meet at its own group barrier, and every block runs its
 * (instance, rank) jobs in one global order.  Each instance draws its own
 * random streams (its index in the batch is part of every RNG counter).
 * The reference runs one problem per process (src/main.cc:15-209); its
 * unused folder loop (src/main.cc:149-207) is the batch front end this
 * replaces.  replicas_per_block in the options caps the replicas of a block
 * (0: the autotuner decides). */
typedef struct pticm_batch pticm_batch;
typedef struct pticm_batch_info {
    uint32_t count, lanes, chunk, jobs, smem_bytes, threads, tuned;
    double makespan_us;     /* predicted device time of one PT step of all instances */
    uint64_t pt_steps, attempts;
    double last_run_ms;
    uint64_t launches;      /* engine launches of pticm_batch_run so far; each is sized from the measured
                               step time to about 0.5 s (the first after a new schedule: one step) */
} pticm_batch_info;
PTICM_API int pticm_batch_create(const pticm_problem* const* problems, uint32_t count, const pticm_opts* o,
                                 pticm_batch** out);
PTICM_API void pticm_batch_destroy(pticm_batch* b);
/* count * nt inverse temperatures, row i for instance i; nc as pticm_set_ladder. */
PTICM_API int pticm_batch_set_ladders(pticm_batch* b, const double* beta, uint32_t nt, int32_t nc);
PTICM_API int pticm_batch_init_states(pticm_batch* b, uint64_t seed);
/* Runs trial_steps PT steps at up to three group sizes per instance, restores
 * the states, and keeps the groups with the shortest predicted makespan. */
PTICM_API int pticm_batch_autotune(pticm_batch* b, uint32_t trial_steps);
PTICM_API int pticm_batch_run(pticm_batch* b, uint64_t pt_steps, uint32_t phase_mask);
PTICM_API int pticm_batch_get_info(pticm_batch* b, pticm_batch_info* info);
/* per instance: blocks, step time (us; measured once tuned), adjacency staged, ICM teams */
PTICM_API int pticm_batch_get_groups(pticm_batch* b, uint32_t* group, double* step_us, int32_t* staged,
                                     int32_t* teams);
/* per instance: best energy (DBL_MAX before any accepted flip) and accepted flips */
PTICM_API int pticm_batch_get_best(pticm_batch* b, double* energy, uint64_t* flips);
PTICM_API int pticm_batch_get_best_state(pticm_batch* b, uint32_t inst, uint8_t* state);
PTICM_API int pticm_batch_get_swap_stats(pticm_batch* b, uint32_t inst, uint64_t* attempts, uint64_t* successes);
PTICM_API int pticm_batch_get_energies(pticm_batch* b, uint32_t inst, int64_t* energy, uint32_t* slot_to_replica);
PTICM_API int pticm_batch_verify(pticm_batch* b, uint64_t* mismatches);
/* Per-slot energy histograms for every instance (as pticm_enable_energy_histograms). */
PTICM_API int pticm_batch_enable_energy_histograms(pticm_batch* b, uint64_t from_step);
/* R rows of nbins counts of one instance (bin b: energy e_lo + 2b); hist may
 * be NULL to query the sizes. */
PTICM_API int pticm_batch_get_energy_histograms(pticm_batch* b, uint32_t inst, uint32_t* hist, int64_t* e_lo,
                                                uint64_t* nbins);
/* The multihistogram ln g of every instance in one device launch (kept for
 * pticm_batch_logdos until the next run). */
PTICM_API int pticm_batch_compute_logdos(pticm_batch* b, double estep);
/* The FP64 multihistogram ln g of one instance from its histograms
 * (temperatures merged over chains; make_histogram and get_partition_iterate,
 * src/cae_estimator.cc:45-69,228-253).  Bin k is energy min_emin + k*estep. */
PTICM_API int pticm_batch_logdos(pticm_batch* b, uint32_t inst, double estep, double* logdos, uint64_t cap,
                                 uint64_t* nbins, double* min_emin, uint64_t* iterations);

/* ------------------------------------------- surrogate ln g(E) network -- */
/* A multilayer perceptron f(features, e) -> ln g / N: 7 inputs, four hidden
 * layers of 256 SiLU units, one linear output; BF16 weights and activations
 * with FP32 accumulation on the tcgen05 tensor cores, FP32 master weights
 * trained with Adam.  Parameters are one flat FP32 vector of
 * pticm_mlp_param_count() values: W1 [256 x 64] (input columns 7.. unused),
 * b1, W2 [256 x 256], b2, W3, b3, W4, b4, w5 [256], b5.  No counterpart in
 * the reference: it serves the learned temperature ladder below. */
typedef struct pticm_mlp pticm_mlp;
PTICM_API int pticm_mlp_create(uint64_t seed, uint32_t batch, pticm_mlp** out);
PTICM_API void pticm_mlp_destroy(pticm_mlp* m);
PTICM_API uint64_t pticm_mlp_param_count(void);
PTICM_API int pticm_mlp_get_params(pticm_mlp* m, float* out);
PTICM_API int pticm_mlp_set_params(pticm_mlp* m, const float* in);
/* Stage n training rows: x (n x 7) and y (n). */
PTICM_API int pticm_mlp_set_data(pticm_mlp* m, const float* x, const float* y, uint64_t n);
/* Mean squared error and its gradient (flat, FP32) on n <= batch rows. */
PTICM_API int pticm_mlp_gradients(pticm_mlp* m, const float* x, const float* y, uint32_t n, float* grads,
                                  float* loss);
/* `steps` Adam steps on shuffled mini-batches; loss_per_step may be NULL. */
PTICM_API int pticm_mlp_train(pticm_mlp* m, const float* x, const float* y, uint64_t n, uint32_t steps, float lr,
                              uint64_t seed, float* loss_per_step);
PTICM_API int pticm_mlp_predict(pticm_mlp* m, const float* x, uint64_t n, float* y);
/* Flat parameter file: "PTICMMLP", u32 version 1, u64 count, count floats. */
PTICM_API int pticm_mlp_save(pticm_mlp* m, const char* path);
PTICM_API int pticm_mlp_load(pticm_mlp* m, const char* path);

/* ------------------------------------------------ learned temperature ladder -- */
/* The network's instance features: ln N / 10, ln M / 12, mean degree / 20,
 * degree std / 10, coupling mean, coupling std; its seventh input is the
 * normalised energy x = E / W, W = sum |J| + sum |h|; its output ln g / N. */
PTICM_API int pticm_problem_features(const pticm_problem* p, float* out6);
/* Predicted ln g on the exact energy levels E = emin + k*estep <= 0.  The
 * levels are those the couplings allow: estep = 2 gcd_i gcd(h_i + sum_j J_ij,
 * 2 J_ij) (4 on +-1 lattices of even degree), in the residue class of the
 * all-up state.  The network output y gives s = ln 2 - E^2/(2 N V) + y/10
 * (V = sum J^2 + sum h^2), ln g = N s. */
PTICM_API int pticm_surrogate_logdos(const pticm_problem* p, pticm_mlp* m, double* logdos, uint64_t cap,
                                     uint64_t* nbins, double* emin, double* estep);
/* get_beta's constant-acceptance walk (src/cae_estimator.cc:367-425) on the
 * predicted ln g: no pilot run.  Arguments as pticm_cae_ladder. */
PTICM_API int pticm_surrogate_ladder(const pticm_problem* p, pticm_mlp* m, double T0, double T1, int inverse,
                                     uint32_t nt, double step_size, double r, double* beta_out, uint32_t* count);
/* Exchange acceptance of each neighbouring pair of a ladder, measured by a
 * PT run (two chains, no ICM) of burn_in + steps steps: acc[k], k < nt-1. */
PTICM_API int pticm_ladder_acceptance(const pticm_problem* p, const double* beta, uint32_t nt, uint64_t seed,
                                      uint64_t steps, uint64_t burn_in, double* acc);
typedef struct pticm_learned_ladder_info {
    uint32_t surrogate_count;   /* temperatures the surrogate ladder placed        */
    int32_t fallback;           /* 1: the multihistogram ladder was used            */
    double mean_deviation;      /* mean |acceptance - r| at the last check          */
    uint32_t rounds;            /* acceptance checks run (1 to 4)                   */
    uint32_t inserted;          /* temperatures the feedback placement added        */
    double first_deviation;     /* mean |acceptance - r| of the surrogate ladder    */
} pticm_learned_ladder_info;
/* The surrogate ladder, checked by pticm_ladder_acceptance over check_steps
 * steps (plus check_steps/4 burn-in).  While its mean |acceptance - r|
 * exceeds tol (0.05), the ladder is placed again from the measured
 * acceptances (pticm_feedback_ladder) and checked again, at most three
 * times (not at all when the first check is off by more than 0.2); if it
 * still deviates, a multihistogram ladder replaces it: from the energy
 * histograms of the last check (two chains at its temperatures) when every
 * pair of it accepted at least 5 % of its exchanges, else from the pilot
 * run of pticm_cae_ladder (2000 samples, 5000 burn-in). */
/* Feedback placement from measured acceptances acc[k] of the gaps of a
 * descending ladder: sigma_k = 2 erfc^-1(acc_k) / (beta_k - beta_{k+1}) (the
 * exchange acceptance of Gaussian energy distributions of width sigma is
 * erfc(dbeta sigma / 2)); the new ladder walks down from beta[0] with
 * dbeta = 2 erfc^-1(r) / sigma until beta_end or nt temperatures.  attempts
 * bounds the acceptance of a gap that saw no exchange. */
PTICM_API int pticm_feedback_ladder(const double* beta, uint32_t count, const double* acc, double attempts, double r,
                                    uint32_t nt, double beta_end, double* beta_out, uint32_t* out_count);
PTICM_API int pticm_learned_ladder(const pticm_problem* p, pticm_mlp* m, double T0, double T1, int inverse,
                                   uint32_t nt, double r, uint64_t check_steps, double tol, uint64_t seed,
                                   double* beta_out, uint32_t* count, pticm_learned_ladder_info* info);

/* The measured shared-memory copy rate of the current GPU (bytes read plus
 * bytes written per second over all SMs, GB/s): one block per SM copies
 * between two 96 KB regions of its shared memory `iters` times.  The peak of
 * the engine's roofline where its data is shared-memory resident.  No
 * counterpart in the reference. */
PTICM_API int pticm_smem_copy_rate(int iters, double* gb_per_s);

/* ----------------------------------------------------------- utilities -- */
PTICM_API const char* pticm_last_error(void);
PTICM_API const char* pticm_version(void);
/* Philox4x32-10 known-answer probe: out[4*i..] = philox(ctr[4*i..], key[2*i..]). */
PTICM_API int pticm_philox_probe(const uint32_t* ctr, const uint32_t* key, uint32_t* out, int count);

#ifdef __cplusplus
}
#endif
#endif
