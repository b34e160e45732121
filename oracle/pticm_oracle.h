/*
 * pticm_oracle.h -- CPU restatement of the PT-ICM reference hot path.
 *
 * TEST INFRASTRUCTURE ONLY.  Only tests/, __graft_entry__.smoke() and the
 * CPU-baseline legs of bench.py may load this library, and only as the checker
 * (or the timed CPU baseline).  The product never links or calls it.
 *
 * Every function restates one reference routine; the citation beside each
 * declaration is the reference file:line it follows (paths relative to the
 * mxburns2022/PT-ICM project root).  The restatement is pinned against the
 * unmodified reference built single-rank (oracle/build_ref.sh): identical
 * printed results for identical seeds (tests/test_oracle_pin.py).
 *
 * Randomness: the reference draws everything from one std::mt19937_64 through
 * libstdc++ (GCC 13.3) distributions.  orc_mt64_* restates the Mersenne
 * Twister (Matsumoto & Nishimura 1998, 64-bit parameters of the C++ standard
 * [rand.predef]); orc_canonical restates generate_canonical<double,53> for a
 * 64-bit engine; orc_uniform_index restates Lemire's nearly-divisionless
 * bounded integer method (ACM TOMACS 29(1), 2019) as libstdc++ applies it;
 * orc_shuffle_u32 and orc_sample_one restate libstdc++'s Fisher-Yates shuffle
 * and selection sampling with its "two indices per draw" batching.
 */
#ifndef PTICM_ORACLE_H
#define PTICM_ORACLE_H

#include <stdint.h>
#include <stddef.h>

#ifdef __cplusplus
extern "C" {
#endif

/* ---------------------------------------------------------------- RNG ---- */
typedef struct orc_mt64 {
    uint64_t x[312];
    int idx;
} orc_mt64;

void orc_mt64_seed(orc_mt64* g, uint64_t seed);           /* include/problem.hh:16 rng_engine(seed) */
uint64_t orc_mt64_next(orc_mt64* g);
double orc_canonical(orc_mt64* g);                         /* include/problem.hh:70 rand_double() */
uint64_t orc_uniform_index(orc_mt64* g, uint64_t range);   /* uniform integer in [0, range) */
void orc_shuffle_u32(uint32_t* a, uint64_t n, orc_mt64* g);/* src/initialization.cc:96-97, src/replica_exchange.cc:89-90 */
int64_t orc_sample_one(uint64_t pop, orc_mt64* g);         /* src/icm.cc:33 std::sample(.., 1, rng) -> position */
int orc_bernoulli_half(orc_mt64* g);                       /* src/initialization.cc:65,70 */

/* ------------------------------------------------------------ Problem ---- */
typedef struct orc_problem orc_problem;

/* Problem::Problem(path, seed, burn_in)  src/problem.cc:183-247 */
int orc_problem_load(const char* path, uint64_t seed, orc_problem** out);
/* Problem(weights, src, dest, linear, seed, burn_in, N, M)  include/problem.hh:43-62 */
int orc_problem_from_coo(int64_t n, int64_t m, const int32_t* src, const int32_t* dst,
                         const double* w, const double* h, uint64_t seed, orc_problem** out);
void orc_problem_free(orc_problem* p);
int64_t orc_problem_n(const orc_problem* p);
int64_t orc_problem_m(const orc_problem* p);
int orc_problem_sparse(const orc_problem* p);
double orc_problem_char_scale(const orc_problem* p);
/* number of directed adjacency entries of the sparse form (2*M for sparse). */
int64_t orc_problem_nnz(const orc_problem* p);
/* adjacency rows in the reference's list order: row_start[n+1], col[nnz], w[nnz].
 * For a dense problem, the nonzero entries of each row in column order. */
void orc_problem_adjacency(const orc_problem* p, int64_t* row_start, int64_t* col, double* w);
void orc_problem_linear(const orc_problem* p, double* h);
orc_mt64* orc_problem_rng(orc_problem* p);

double orc_energy(const orc_problem* p, const uint8_t* s);                  /* src/problem.cc:124-142 */
double orc_maxcut(const orc_problem* p, const uint8_t* s);                  /* src/problem.cc:145-162 */
double orc_calculate_dE(const orc_problem* p, const uint8_t* s, double* dE);/* src/problem.cc:33-63 */
void orc_incremental_dE(const orc_problem* p, double* dE, const uint8_t* s, int64_t i); /* src/problem.cc:164-181 */

/* ------------------------------------------------------------ Replica ---- */
/* Replica::sweep on one replica, sequential site order 0..N-1
 * (src/replica.cc:5-38).  Uniforms come from p's engine.  `trace_u`, when not
 * NULL, receives every uniform consumed (capacity `cap`, count in *n_used).
 * best_* follow src/replica.cc:23-27.  Returns accepted flips in this call. */
uint64_t orc_sweep(orc_problem* p, double beta, uint8_t* s, double* dE, double* energy,
                   double* best_E, uint64_t* best_sweep, uint8_t* best_state,
                   uint64_t sweep_counter, double* trace_u, uint64_t cap, uint64_t* n_used);

/* Same sweep but consuming a caller-supplied uniform stream instead of an
 * engine (the replay contract).  *pos advances by the uniforms consumed. */
uint64_t orc_sweep_stream(const orc_problem* p, double beta, uint8_t* s, double* dE,
                          double* energy, double* best_E, uint64_t* best_sweep,
                          uint8_t* best_state, uint64_t sweep_counter,
                          const double* u, uint64_t n_u, uint64_t* pos);

/* ------------------------------------------------------------- Ladder ---- */
void orc_beta_linspace(double* beta, double T0, double T1, uint64_t nt, int inverse); /* src/utils.cc:6-22 */

/* ------------------------------------------------------------ Solver ----- */
typedef struct orc_params {
    uint64_t seed;
    uint64_t Nt;            /* temperatures per chain (-r)                       */
    uint64_t pts;           /* PT steps (--pts)                                  */
    uint64_t sweeps;        /* sweeps per PT step (--sweeps)                     */
    uint64_t pre_samples;   /* --preprocess-samples                              */
    uint64_t pilot_burn_in; /* BURN_IN of src/cae_estimator.cc:74 (5000 there)   */
    double T0, T1;
    double pre_step;        /* --preprocess-stepsize                             */
    int inverse, preprocess, icm;
} orc_params;

/* Everything `solve` prints (src/solver.cc:151-163) plus final replica data. */
typedef struct orc_result {
    uint64_t Nt;            /* after --preprocess this is the selected count     */
    uint32_t Nc;            /* ICM pairs (src/initialization.cc:158-164)         */
    double beta[2048];      /* ladder, 2*Nt entries                              */
    uint32_t swap_attempts[2048];
    uint32_t swap_successes[2048];
    uint64_t swaps;
    double best_energy;
    uint64_t best_sweep;
    double best_state_energy;
    double best_maxcut;
    uint64_t flips;         /* as printed: int-typed accumulate (src/mpi_utils.cc:168) */
    uint64_t flips_u64;     /* the untruncated sum                               */
    double char_scale;
} orc_result;

/* Optional trace of every random decision, for the device replay. */
typedef struct orc_trace orc_trace;
orc_trace* orc_trace_new(void);
/* A trace that records only the slot energies after the sweeps of each step
 * (no uniforms or decisions): statistics of long runs. */
orc_trace* orc_trace_new_energy_only(void);
void orc_trace_free(orc_trace* t);
/* accessors (sizes first, then copies into caller buffers) */
uint64_t orc_trace_n_uniforms(const orc_trace* t);
uint64_t orc_trace_n_sweeps(const orc_trace* t);        /* entries of the offsets table - 1 */
uint64_t orc_trace_n_exchange(const orc_trace* t);
uint64_t orc_trace_n_icm(const orc_trace* t);
uint64_t orc_trace_n_init(const orc_trace* t);
uint64_t orc_trace_n_energy(const orc_trace* t);
void orc_trace_copy(const orc_trace* t, double* uniforms, uint64_t* sweep_offsets,
                    int32_t* xchg_pair, double* xchg_logu, int64_t* icm_seed,
                    uint8_t* init_states, double* step_energy);

/* solve() of src/solver.cc:16-166 on one rank.  `replica_states` (2*Nt*N
 * bytes, may be NULL) receives the final spins, `best_state` (N bytes) the
 * reported best state, `final_energy` (2*Nt) the final energies. */
int orc_solve(orc_problem* p, const orc_params* prm, orc_result* res,
              uint8_t* best_state, uint8_t* replica_states, double* final_energy,
              orc_trace* trace);

/* ------------------------------------------------------- One ICM pair ---- */
/* xor_icm's overlap (src/icm.cc:8-31) without its seed draw: negates s1 when
 * more than N/2 sites differ; writes the differing sites ascending to
 * `sites` (N entries) and returns their count. */
int64_t orc_overlap(const orc_problem* p, uint8_t* s1, const uint8_t* s2, int64_t* sites);
/* bfs_icm (src/icm.cc:37-72): flips the seed's cluster of differing sites in
 * both states. */
void orc_bfs_icm(const orc_problem* p, int64_t seed, uint8_t* s1, uint8_t* s2);

/* orc_solve without outputs beyond `res`, timing its main loop from PT step
 * `timed_from` on: *timed_s receives the wall seconds of steps timed_from ..
 * pts-1 (the CPU baseline times a run past its random start). */
int orc_solve_timed(orc_problem* p, const orc_params* prm, orc_result* res, uint64_t timed_from, double* timed_s);

/* ---------------------------------------------- Multihistogram (CAE) ----- */
/* Restatements of src/cae_estimator.cc: the pilot run (gather_samples :76-151),
 * histograms (:45-69), log-space DOS fixed point (:155-253) and the greedy
 * constant-acceptance ladder walk (get_beta :295-428). */
double orc_logplusexp2(double l1, double l2);                                 /* :30-36 */
double orc_partition_func(const double* logdos, uint64_t nb, double beta, double emin, double estep); /* :155-170 */
/* calculate_dos (:172-226): hist is Nt rows, row j of length hist_len[j] at
 * hist_off[j] in `hist`.  Writes nbins=ceil((max_emax-min_emin)/estep) values. */
uint64_t orc_calculate_dos(const uint32_t* hist, const uint64_t* hist_off, const uint64_t* hist_len,
                           uint64_t nt, const double* logZ, const double* emin_values,
                           const double* beta_hist, double estep, double min_emin, double max_emax,
                           uint64_t n, double* logdos);
/* get_partition_iterate (:228-253); returns iterations, logdos sized as above. */
uint64_t orc_partition_iterate(const uint32_t* hist, const uint64_t* hist_off, const uint64_t* hist_len,
                               uint64_t nt, const double* beta_hist, const double* emin_values,
                               double estep, uint64_t n, double max_emax,
                               double* logdos, double* logZ);
double orc_acceptance_rate(const double* logdos, uint64_t nb, const double* p1, const double* p2,
                           double beta1, double beta2, double estep, double emin); /* :262-293 */
/* CAE walk of get_beta (:367-425) from a converged logdos; returns the count. */
uint64_t orc_cae_walk(const double* logdos, uint64_t nb, double min_emin, double estep,
                      double beta_start, double beta_end, double step_size, double r,
                      uint64_t num_temps, double* beta_out);
/* Whole get_beta (:295-428) including the pilot run on p's engine.  Returns
 * the selected temperature count; beta_out holds >= num_temps entries.
 * Optional outputs (may be NULL): histogram data for cross-checking. */
uint64_t orc_get_beta(orc_problem* p, double T0, double T1, int inverse, uint64_t num_temps,
                      double estep, double step_size, double r, uint64_t num_samples,
                      uint64_t burn_in, double* beta_out,
                      double* hist_betas_out, double* emin_out, double* emax_out);

/* The pilot run and histograms of get_beta on a given hist_betas ladder:
 * writes up to hist_cap counts, returns the total; see orc_get_beta. */
uint64_t orc_pilot(orc_problem* p, const double* hist_betas, uint64_t nt, double estep, uint64_t num_samples,
                   uint64_t burn_in, uint32_t* hist_out, uint64_t hist_cap, uint64_t* hist_off, uint64_t* hist_len,
                   double* emin, double* emax, uint64_t* n_out);

#ifdef __cplusplus
}
#endif
#endif
