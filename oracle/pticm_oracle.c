/*
 * pticm_oracle.c -- CPU restatement of the PT-ICM reference hot path.
 *
 * TEST INFRASTRUCTURE ONLY (see pticm_oracle.h): the checker for the device
 * kernels and the "port" CPU baseline of bench.py.  Never linked by the
 * product.  Each routine cites the reference file:line it restates.
 */
#define _GNU_SOURCE
#include "pticm_oracle.h"

#include <float.h>
#include <math.h>
#include <stdio.h>
#include <stdlib.h>
#include <string.h>
#include <time.h>

/* ===================================================================== RNG */
/* Mersenne Twister, 64-bit word size; parameters of std::mt19937_64. */
#define MT_N 312
#define MT_M 156
#define MT_UPPER 0xFFFFFFFF80000000ULL
#define MT_LOWER 0x000000007FFFFFFFULL

void orc_mt64_seed(orc_mt64* g, uint64_t seed) {
    g->x[0] = seed;
    for (int i = 1; i < MT_N; i++) {
        uint64_t p = g->x[i - 1];
        g->x[i] = 6364136223846793005ULL * (p ^ (p >> 62)) + (uint64_t)i;
    }
    g->idx = MT_N;
}

static void mt_regen(orc_mt64* g) {
    for (int i = 0; i < MT_N; i++) {
        uint64_t y = (g->x[i] & MT_UPPER) | (g->x[(i + 1) % MT_N] & MT_LOWER);
        uint64_t v = g->x[(i + MT_M) % MT_N] ^ (y >> 1);
        if (y & 1ULL) v ^= 0xB5026F5AA96619E9ULL;
        g->x[i] = v;
    }
    g->idx = 0;
}

uint64_t orc_mt64_next(orc_mt64* g) {
    if (g->idx >= MT_N) mt_regen(g);
    uint64_t z = g->x[g->idx++];
    z ^= (z >> 29) & 0x5555555555555555ULL;
    z ^= (z << 17) & 0x71D67FFFEDA60000ULL;
    z ^= (z << 37) & 0xFFF7EEE000000000ULL;
    z ^= z >> 43;
    return z;
}

/* A 64-bit engine fills 53 mantissa bits with one draw: u = double(x) / 2^64,
 * clamped below 1 (the round-to-nearest conversion can reach 2^64). */
double orc_canonical(orc_mt64* g) {
    double u = (double)orc_mt64_next(g) / 18446744073709551616.0;
    if (u >= 1.0) u = nextafter(1.0, 0.0);
    return u;
}

/* Bounded integer in [0, range), range >= 1, by Lemire's multiply-and-reject:
 * take the high word of x*range, rejecting low words below 2^64 mod range. */
uint64_t orc_uniform_index(orc_mt64* g, uint64_t range) {
    unsigned __int128 prod = (unsigned __int128)orc_mt64_next(g) * range;
    uint64_t low = (uint64_t)prod;
    if (low < range) {
        uint64_t thresh = (0 - range) % range;
        while (low < thresh) {
            prod = (unsigned __int128)orc_mt64_next(g) * range;
            low = (uint64_t)prod;
        }
    }
    return (uint64_t)(prod >> 64);
}

/* Fisher-Yates from the front.  When n*n fits the engine range, two swap
 * positions come from one draw over [0, b*(b+1)) split as (x / (b+1), x % (b+1)),
 * after one single-bit draw that makes the remaining count even. */
void orc_shuffle_u32(uint32_t* a, uint64_t n, orc_mt64* g) {
    if (n == 0) return;
    uint64_t i = 1;
    if (UINT64_MAX / n >= n) {
        if (n % 2 == 0) {
            uint64_t j = orc_uniform_index(g, 2);
            uint32_t t = a[i]; a[i] = a[j]; a[j] = t;
            i++;
        }
        while (i != n) {
            uint64_t b = i + 1;
            uint64_t x = orc_uniform_index(g, b * (b + 1));
            uint64_t p0 = x / (b + 1), p1 = x % (b + 1);
            uint32_t t = a[i]; a[i] = a[p0]; a[p0] = t;
            i++;
            t = a[i]; a[i] = a[p1]; a[p1] = t;
            i++;
        }
        return;
    }
    for (; i != n; i++) {
        uint64_t j = orc_uniform_index(g, i + 1);
        uint32_t t = a[i]; a[i] = a[j]; a[j] = t;
    }
}

/* Selection sampling of one element out of `pop`: walk the population, keeping
 * element k with probability 1/(remaining); two decisions per draw while at
 * least two elements remain, a final single draw otherwise.  Returns the
 * position of the chosen element, -1 for an empty population. */
int64_t orc_sample_one(uint64_t pop, orc_mt64* g) {
    if (pop == 0) return -1;
    uint64_t unsampled = pop;
    uint64_t pos = 0;
    if (UINT64_MAX / unsampled >= unsampled) {
        while (unsampled >= 2) {
            uint64_t b0 = unsampled, b1 = unsampled - 1;
            uint64_t x = orc_uniform_index(g, b0 * b1);
            uint64_t first = x / b1, second = x % b1;
            --unsampled;
            if (first < 1) return (int64_t)pos;
            ++pos;
            --unsampled;
            if (second < 1) return (int64_t)pos;
            ++pos;
        }
    }
    for (;; ++pos) {
        --unsampled;
        if (orc_uniform_index(g, unsampled + 1) < 1) return (int64_t)pos;
    }
}

int orc_bernoulli_half(orc_mt64* g) { return orc_canonical(g) < 0.5; }

/* ================================================================= Problem */
struct orc_problem {
    int64_t n, m;
    int sparse;
    int64_t* row;   /* sparse: n+1 */
    int64_t* col;   /* sparse: nnz */
    double* w;      /* sparse: nnz ; dense: n*n */
    double* h;
    double char_scale;
    orc_mt64 rng;
};

static inline int sgn(uint8_t b) { return (int)b * 2 - 1; } /* include/utils.hh:78-81 */

static orc_problem* prob_alloc(int64_t n) {
    orc_problem* p = (orc_problem*)calloc(1, sizeof(orc_problem));
    p->n = n;
    p->h = (double*)calloc((size_t)(n > 0 ? n : 1), sizeof(double));
    return p;
}

void orc_problem_free(orc_problem* p) {
    if (!p) return;
    free(p->row); free(p->col); free(p->w); free(p->h); free(p);
}

/* Build the adjacency lists in the reference's push_back order from a COO
 * list: line k appends (u->v) to u's list, then (v->u) to v's list. */
static void build_sparse(orc_problem* p, int64_t m, const int64_t* u, const int64_t* v, const double* w) {
    int64_t n = p->n;
    p->sparse = 1;
    p->row = (int64_t*)calloc((size_t)n + 1, sizeof(int64_t));
    for (int64_t k = 0; k < m; k++) { p->row[u[k] + 1]++; p->row[v[k] + 1]++; }
    for (int64_t i = 0; i < n; i++) p->row[i + 1] += p->row[i];
    int64_t nnz = p->row[n];
    p->col = (int64_t*)malloc((size_t)(nnz > 0 ? nnz : 1) * sizeof(int64_t));
    p->w = (double*)malloc((size_t)(nnz > 0 ? nnz : 1) * sizeof(double));
    int64_t* fill = (int64_t*)malloc((size_t)(n > 0 ? n : 1) * sizeof(int64_t));
    for (int64_t i = 0; i < n; i++) fill[i] = p->row[i];
    for (int64_t k = 0; k < m; k++) {
        int64_t a = fill[u[k]]++; p->col[a] = v[k]; p->w[a] = w[k];
        int64_t b = fill[v[k]]++; p->col[b] = u[k]; p->w[b] = w[k];
    }
    free(fill);
}

/* Parse one unsigned integer the way `istream >> uint64_t` does for the
 * inputs the reference reads: skip white space, read decimal digits. */
static int parse_u64(const char** s, const char* end, uint64_t* out) {
    const char* c = *s;
    while (c < end && (*c == ' ' || *c == '\t' || *c == '\r' || *c == '\n' || *c == '\v' || *c == '\f')) c++;
    if (c >= end || *c < '0' || *c > '9') return 0;
    uint64_t v = 0;
    while (c < end && *c >= '0' && *c <= '9') { v = v * 10 + (uint64_t)(*c - '0'); c++; }
    *s = c;
    *out = v;
    return 1;
}

/* `istream >> double` on the rest of a line: white space, then a number; a
 * failed extraction yields 0.0 (C++11 semantics). */
static double parse_double_rest(const char* c, const char* end) {
    char buf[128];
    while (c < end && (*c == ' ' || *c == '\t' || *c == '\r' || *c == '\v' || *c == '\f')) c++;
    size_t len = (size_t)(end - c);
    if (len == 0) return 0.0;
    if (len > sizeof(buf) - 1) len = sizeof(buf) - 1;
    memcpy(buf, c, len);
    buf[len] = 0;
    char* e = NULL;
    double v = strtod(buf, &e);
    if (e == buf) return 0.0;
    return v;
}

/* src/problem.cc:183-247.  Error codes: 1 unreadable file, 2 malformed line,
 * 3 vertex index out of range. */
int orc_problem_load(const char* path, uint64_t seed, orc_problem** out) {
    *out = NULL;
    FILE* f = fopen(path, "rb");
    if (!f) return 1;
    fseek(f, 0, SEEK_END);
    long sz = ftell(f);
    fseek(f, 0, SEEK_SET);
    char* buf = (char*)malloc((size_t)sz + 1);
    if (fread(buf, 1, (size_t)sz, f) != (size_t)sz) { fclose(f); free(buf); return 1; }
    fclose(f);
    buf[sz] = 0;
    const char* c = buf;
    const char* end = buf + sz;
    int is_ising = strstr(path, ".ising") != NULL;
    int zero_based = strstr(path, ".gset") != NULL || is_ising;
    uint64_t N = 0, M = 0, num_linear = 0;
    if (!parse_u64(&c, end, &N)) { free(buf); return 2; }
    if (is_ising && !parse_u64(&c, end, &num_linear)) { free(buf); return 2; }
    if (!parse_u64(&c, end, &M)) { free(buf); return 2; }
    orc_problem* p = prob_alloc((int64_t)N);
    orc_mt64_seed(&p->rng, seed);
    p->m = (int64_t)M;
    uint64_t pairs = N * (N - 1) / 2;
    int sparse = ((double)M / (double)pairs) < 0.1;
    int64_t cap = 1024, cnt = 0;
    int64_t* eu = (int64_t*)malloc((size_t)cap * sizeof(int64_t));
    int64_t* ev = (int64_t*)malloc((size_t)cap * sizeof(int64_t));
    double* ew = (double*)malloc((size_t)cap * sizeof(double));
    int64_t off = zero_based ? 0 : -1;
    uint64_t nlin = 0;
    double sum = 0, sqsum = 0;
    double w = 0.0;
    int rc = 0;
    if (!sparse) {
        p->w = (double*)calloc((size_t)N * (size_t)N, sizeof(double));
    }
    while (c < end) {
        const char* ls = c;
        const char* le = memchr(c, '\n', (size_t)(end - c));
        if (!le) le = end;
        c = (le < end) ? le + 1 : end;
        if (le - ls <= 1) continue;
        const char* q = ls;
        uint64_t u = 0, v = 0;
        if (nlin < num_linear) {
            if (!parse_u64(&q, le, &u)) { rc = 2; break; }
            int64_t ui = (int64_t)u + off;
            if (ui < 0 || ui >= (int64_t)N) { rc = 3; break; }
            p->h[ui] = parse_double_rest(q, le);
            nlin++;
            continue;
        }
        if (!parse_u64(&q, le, &u) || !parse_u64(&q, le, &v)) { rc = 2; break; }
        int64_t ui = (int64_t)u + off, vi = (int64_t)v + off;
        if (ui < 0 || vi < 0 || ui >= (int64_t)N || vi >= (int64_t)N) { rc = 3; break; }
        if (q == le) w = 1.0;              /* stream at eof after v */
        else w = parse_double_rest(q, le); /* else `>> w`, 0.0 when nothing parses */
        sum += w;
        sqsum += w * w;
        if (sparse) {
            if (cnt == cap) {
                cap *= 2;
                eu = (int64_t*)realloc(eu, (size_t)cap * sizeof(int64_t));
                ev = (int64_t*)realloc(ev, (size_t)cap * sizeof(int64_t));
                ew = (double*)realloc(ew, (size_t)cap * sizeof(double));
            }
            eu[cnt] = ui; ev[cnt] = vi; ew[cnt] = w; cnt++;
        } else {
            p->w[ui * (int64_t)N + vi] = w;
            p->w[vi * (int64_t)N + ui] = w;
        }
    }
    free(buf);
    if (rc) { free(eu); free(ev); free(ew); orc_problem_free(p); return rc; }
    if (sparse) build_sparse(p, cnt, eu, ev, ew);
    free(eu); free(ev); free(ew);
    double variance = sqsum / (double)M - (sum / (double)M * sum / (double)M);
    /* std::max(mean, variance) keeps the first argument on ties */
    p->char_scale = (sum / (double)M >= variance) ? sum / (double)M : variance;
    *out = p;
    return 0;
}

int orc_problem_from_coo(int64_t n, int64_t m, const int32_t* src, const int32_t* dst,
                         const double* w, const double* h, uint64_t seed, orc_problem** out) {
    orc_problem* p = prob_alloc(n);
    orc_mt64_seed(&p->rng, seed);
    p->m = m;
    int64_t* u = (int64_t*)malloc((size_t)(m > 0 ? m : 1) * sizeof(int64_t));
    int64_t* v = (int64_t*)malloc((size_t)(m > 0 ? m : 1) * sizeof(int64_t));
    double sum = 0, sq = 0;
    for (int64_t k = 0; k < m; k++) {
        if (src[k] < 0 || src[k] >= n || dst[k] < 0 || dst[k] >= n) { free(u); free(v); orc_problem_free(p); *out = NULL; return 3; }
        u[k] = src[k]; v[k] = dst[k]; sum += w[k]; sq += w[k] * w[k];
    }
    build_sparse(p, m, u, v, w);
    free(u); free(v);
    if (h) memcpy(p->h, h, (size_t)n * sizeof(double));
    double variance = m ? sq / (double)m - (sum / (double)m * sum / (double)m) : 0.0;
    double mean = m ? sum / (double)m : 0.0;
    p->char_scale = mean >= variance ? mean : variance;
    *out = p;
    return 0;
}

int64_t orc_problem_n(const orc_problem* p) { return p->n; }
int64_t orc_problem_m(const orc_problem* p) { return p->m; }
int orc_problem_sparse(const orc_problem* p) { return p->sparse; }
double orc_problem_char_scale(const orc_problem* p) { return p->char_scale; }
orc_mt64* orc_problem_rng(orc_problem* p) { return &p->rng; }

int64_t orc_problem_nnz(const orc_problem* p) {
    if (p->sparse) return p->row[p->n];
    int64_t k = 0;
    for (int64_t i = 0; i < p->n; i++)
        for (int64_t j = 0; j < p->n; j++)
            if (i != j && p->w[i * p->n + j] != 0.0) k++;
    return k;
}

void orc_problem_adjacency(const orc_problem* p, int64_t* row_start, int64_t* col, double* w) {
    if (p->sparse) {
        memcpy(row_start, p->row, (size_t)(p->n + 1) * sizeof(int64_t));
        memcpy(col, p->col, (size_t)p->row[p->n] * sizeof(int64_t));
        memcpy(w, p->w, (size_t)p->row[p->n] * sizeof(double));
        return;
    }
    int64_t k = 0;
    for (int64_t i = 0; i < p->n; i++) {
        row_start[i] = k;
        for (int64_t j = 0; j < p->n; j++)
            if (i != j && p->w[i * p->n + j] != 0.0) { col[k] = j; w[k] = p->w[i * p->n + j]; k++; }
    }
    row_start[p->n] = k;
}

void orc_problem_linear(const orc_problem* p, double* h) { memcpy(h, p->h, (size_t)p->n * sizeof(double)); }

double orc_energy(const orc_problem* p, const uint8_t* s) {
    double ene = 0.0;
    int64_t N = p->n;
    for (int64_t i = 0; i < N; i++) {
        int ival = sgn(s[i]);
        ene += ival * p->h[i];
        if (p->sparse) {
            for (int64_t a = p->row[i]; a < p->row[i + 1]; a++)
                ene += 0.5 * ival * sgn(s[p->col[a]]) * p->w[a];
        } else {
            const double* r = p->w + i * N;
            for (int64_t j = i + 1; j < N; j++) ene += ival * sgn(s[j]) * r[j];
        }
    }
    return ene;
}

double orc_maxcut(const orc_problem* p, const uint8_t* s) {
    double cut = 0.0;
    int64_t N = p->n;
    for (int64_t i = 0; i < N; i++) {
        int ival = s[i];
        if (p->sparse) {
            for (int64_t a = p->row[i]; a < p->row[i + 1]; a++)
                cut += ival != s[p->col[a]] ? 0.5 * p->w[a] : 0;
        } else {
            const double* r = p->w + i * N;
            for (int64_t j = i + 1; j < N; j++) cut += ival != s[j] ? r[j] : 0;
        }
    }
    return cut;
}

double orc_calculate_dE(const orc_problem* p, const uint8_t* s, double* dE) {
    double ene = 0.0, term;
    int64_t N = p->n;
    for (int64_t i = 0; i < N; i++) {
        dE[i] = -2 * p->h[i] * sgn(s[i]);
        ene += p->h[i] * sgn(s[i]);
    }
    for (int64_t i = 0; i < N; i++) {
        int ival = sgn(s[i]);
        if (p->sparse) {
            for (int64_t a = p->row[i]; a < p->row[i + 1]; a++) {
                term = ival * sgn(s[p->col[a]]) * p->w[a];
                ene += term / 2;
                dE[i] -= 2 * term;
            }
        } else {
            const double* r = p->w + i * N;
            for (int64_t j = 0; j < N; j++) {
                if (i == j) continue;
                term = ival * sgn(s[j]) * r[j];
                ene += term / 2;
                dE[i] -= 2 * term;
            }
        }
    }
    return ene;
}

void orc_incremental_dE(const orc_problem* p, double* dE, const uint8_t* s, int64_t index) {
    dE[index] *= -1;
    int ival = sgn(s[index]);
    if (p->sparse) {
        for (int64_t a = p->row[index]; a < p->row[index + 1]; a++)
            dE[p->col[a]] += 4 * ival * sgn(s[p->col[a]]) * p->w[a];
    } else {
        const double* r = p->w + index * p->n;
        for (int64_t j = 0; j < p->n; j++) {
            if (j == index) continue;
            dE[j] += 4 * ival * sgn(s[j]) * r[j];
        }
    }
}

/* ================================================================= Replica */
/* mh_accept (src/replica.cc:18-29) */
static inline void mh_accept(const orc_problem* p, uint8_t* s, double* dE, double* energy, int64_t i,
                             double* best_E, uint64_t* best_sweep, uint8_t* best_state, uint64_t sweep_counter) {
    *energy += dE[i];
    orc_incremental_dE(p, dE, s, i);
    s[i] = !s[i];
    if (*energy < *best_E) {
        *best_E = *energy;
        if (best_state) memcpy(best_state, s, (size_t)p->n);
        *best_sweep = sweep_counter;
    }
}

uint64_t orc_sweep(orc_problem* p, double beta, uint8_t* s, double* dE, double* energy,
                   double* best_E, uint64_t* best_sweep, uint8_t* best_state,
                   uint64_t sweep_counter, double* trace_u, uint64_t cap, uint64_t* n_used) {
    uint64_t flips = 0, used = 0;
    for (int64_t i = 0; i < p->n; i++) {
        int acc;
        if (dE[i] <= 0) {
            acc = 1;
        } else {
            double boltzmann = exp(-beta * dE[i]);
            double u = orc_canonical(&p->rng);
            if (trace_u && used < cap) trace_u[used] = u;
            used++;
            acc = u < boltzmann;
        }
        if (acc) {
            mh_accept(p, s, dE, energy, i, best_E, best_sweep, best_state, sweep_counter);
            flips++;
        }
    }
    if (n_used) *n_used = used;
    return flips;
}

uint64_t orc_sweep_stream(const orc_problem* p, double beta, uint8_t* s, double* dE,
                          double* energy, double* best_E, uint64_t* best_sweep,
                          uint8_t* best_state, uint64_t sweep_counter,
                          const double* u, uint64_t n_u, uint64_t* pos) {
    uint64_t flips = 0;
    for (int64_t i = 0; i < p->n; i++) {
        int acc;
        if (dE[i] <= 0) {
            acc = 1;
        } else {
            double boltzmann = exp(-beta * dE[i]);
            double x = (*pos < n_u) ? u[*pos] : 1.0;
            (*pos)++;
            acc = x < boltzmann;
        }
        if (acc) {
            mh_accept(p, s, dE, energy, i, best_E, best_sweep, best_state, sweep_counter);
            flips++;
        }
    }
    return flips;
}

/* ================================================================== Ladder */
void orc_beta_linspace(double* temps, double T0, double T1, uint64_t num_temp, int inverse) {
    double step, curr;
    if (inverse) {
        step = T1 < T0 ? (T0 - T1) / (double)(num_temp - 1) : (T1 - T0) / (double)(num_temp - 1);
        curr = T1 < T0 ? T1 : T0;
    } else {
        step = T1 < T0 ? (1 / T1 - 1 / T0) / (double)(num_temp - 1) : (1 / T0 - 1 / T1) / (double)(num_temp - 1);
        curr = T1 < T0 ? 1 / T0 : 1 / T1;
    }
    for (uint64_t i = 0; i < num_temp; i++) {
        temps[i] = curr;
        curr += step;
    }
}

/* =================================================================== Trace */
typedef struct { void* p; uint64_t n, cap; size_t el; } vec_t;
static void vpush(vec_t* v, const void* x) {
    if (v->n == v->cap) {
        v->cap = v->cap ? v->cap * 2 : 1024;
        v->p = realloc(v->p, v->cap * v->el);
    }
    memcpy((char*)v->p + v->n * v->el, x, v->el);
    v->n++;
}

struct orc_trace {
    vec_t u;        /* double  : sweep uniforms                              */
    vec_t off;      /* uint64  : start offset of each (step, sweep, replica) */
    vec_t xk;       /* int32   : exchange pair slot                          */
    vec_t xlu;      /* double  : log(u) of each exchange attempt             */
    vec_t icm;      /* int64   : ICM seed site, -1 when the pair is equal    */
    vec_t init;     /* uint8   : initial states, replica-major               */
    vec_t energy;   /* double  : slot energies after the sweeps of each step */
    int energy_only;/* record the slot energies alone (long runs)            */
};

orc_trace* orc_trace_new(void) {
    orc_trace* t = (orc_trace*)calloc(1, sizeof(orc_trace));
    t->u.el = sizeof(double); t->off.el = sizeof(uint64_t); t->xk.el = sizeof(int32_t);
    t->xlu.el = sizeof(double); t->icm.el = sizeof(int64_t); t->init.el = 1; t->energy.el = sizeof(double);
    return t;
}
orc_trace* orc_trace_new_energy_only(void) {
    orc_trace* t = orc_trace_new();
    t->energy_only = 1;
    return t;
}
void orc_trace_free(orc_trace* t) {
    if (!t) return;
    free(t->u.p); free(t->off.p); free(t->xk.p); free(t->xlu.p); free(t->icm.p); free(t->init.p); free(t->energy.p);
    free(t);
}
uint64_t orc_trace_n_uniforms(const orc_trace* t) { return t->u.n; }
uint64_t orc_trace_n_sweeps(const orc_trace* t) { return t->off.n ? t->off.n - 1 : 0; }
uint64_t orc_trace_n_exchange(const orc_trace* t) { return t->xk.n; }
uint64_t orc_trace_n_icm(const orc_trace* t) { return t->icm.n; }
uint64_t orc_trace_n_init(const orc_trace* t) { return t->init.n; }
uint64_t orc_trace_n_energy(const orc_trace* t) { return t->energy.n; }
void orc_trace_copy(const orc_trace* t, double* uniforms, uint64_t* sweep_offsets,
                    int32_t* xchg_pair, double* xchg_logu, int64_t* icm_seed,
                    uint8_t* init_states, double* step_energy) {
    if (uniforms && t->u.n) memcpy(uniforms, t->u.p, t->u.n * t->u.el);
    if (sweep_offsets && t->off.n) memcpy(sweep_offsets, t->off.p, t->off.n * t->off.el);
    if (xchg_pair && t->xk.n) memcpy(xchg_pair, t->xk.p, t->xk.n * t->xk.el);
    if (xchg_logu && t->xlu.n) memcpy(xchg_logu, t->xlu.p, t->xlu.n * t->xlu.el);
    if (icm_seed && t->icm.n) memcpy(icm_seed, t->icm.p, t->icm.n * t->icm.el);
    if (init_states && t->init.n) memcpy(init_states, t->init.p, t->init.n);
    if (step_energy && t->energy.n) memcpy(step_energy, t->energy.p, t->energy.n * t->energy.el);
}

/* ================================================================== Solver */
typedef struct {
    orc_problem* p;
    uint64_t Nt, R, N;
    double* beta_values;   /* 2Nt slot values                         */
    uint32_t* bidx;        /* slot -> replica                         */
    double* rep_beta;      /* replica -> its beta                     */
    uint8_t* chain;        /* replica -> chain                        */
    uint8_t* s;            /* R*N                                     */
    double* dE;            /* R*N                                     */
    double* E;             /* R                                       */
    double* Eg;            /* energies gathered after the sweeps      */
    uint32_t* flips;       /* R (uint32 like Replica::flips)          */
    double* bestE;
    uint64_t* bestSweep;
    uint8_t* bestS;        /* R*N                                     */
    uint64_t* sweepCtr;
    uint32_t* order1;
    uint32_t* order2;
    uint32_t xi;
    uint32_t* att;
    uint32_t* succ;
    uint64_t swaps;
    orc_trace* tr;
} pt_t;

/* get_replica (src/mpi_utils.cc:215-226): first replica of `chain` whose beta
 * equals `beta` within 1e-10. */
static int64_t get_replica(pt_t* w, double beta, int chain) {
    for (uint64_t i = 0; i < w->R; i++)
        if (fabs(beta - w->rep_beta[i]) < 1e-10 && chain == w->chain[i]) return (int64_t)i;
    return -1;
}

/* do_replica_exchange_local (src/replica_exchange.cc:103-125) */
static void exchange_local(pt_t* w, double beta_old, double beta_new, int chain) {
    for (uint64_t j = 0; j < w->R; j++) {
        if (fabs(w->rep_beta[j] - beta_new) < 1e-10 && w->chain[j] == chain) w->rep_beta[j] = beta_old;
        else if (fabs(w->rep_beta[j] - beta_old) < 1e-10 && w->chain[j] == chain) w->rep_beta[j] = beta_new;
    }
}

/* try_replica_exchange (src/replica_exchange.cc:5-100), rank 0 owning all. */
static void try_exchange(pt_t* w, int chain_index) {
    uint64_t Nt = w->Nt;
    uint64_t k = w->order1[w->xi] + (chain_index ? Nt : 0);
    w->att[k]++;
    uint32_t r1 = w->bidx[k], r2 = w->bidx[k + 1];
    double bl = w->beta_values[k], bh = w->beta_values[k + 1];
    double dBeta = bl - bh;
    double dE = w->Eg[r1] - w->Eg[r2];
    double logb = dBeta * dE;
    double rnd = log(orc_canonical(&w->p->rng));
    if (w->tr) { int32_t kk = (int32_t)k; vpush(&w->tr->xk, &kk); vpush(&w->tr->xlu, &rnd); }
    if ((dE * dBeta) > 0 || rnd < logb) {
        w->succ[k]++;
        w->swaps++;
        exchange_local(w, bl, bh, chain_index);
        uint32_t t = w->bidx[k]; w->bidx[k] = w->bidx[k + 1]; w->bidx[k + 1] = t;
    }
    w->xi++;
    if (w->xi == Nt - 1) {
        w->xi = 0;
        orc_shuffle_u32(w->order1, Nt - 1, &w->p->rng);
        orc_shuffle_u32(w->order2, Nt - 1, &w->p->rng);
    }
}

/* xor_icm (src/icm.cc:8-35) */
static int64_t xor_icm(pt_t* w, uint8_t* s1, const uint8_t* s2, int64_t* tmp) {
    uint64_t N = w->N, cnt = 0;
    for (uint64_t j = 0; j < N; j++) if (s1[j] ^ s2[j]) tmp[cnt++] = (int64_t)j;
    if (cnt > N / 2) {
        cnt = 0;
        for (uint64_t j = 0; j < N; j++) {
            s1[j] = !s1[j];
            if (s1[j] != s2[j]) tmp[cnt++] = (int64_t)j;
        }
    }
    if (cnt == 0) return -1;
    int64_t pos = orc_sample_one(cnt, &w->p->rng);
    return tmp[pos];
}

/* bfs_icm (src/icm.cc:37-72): depth-first growth of the seed's cluster of
 * differing sites, flipped in both states. */
static void bfs_icm(const orc_problem* p, int64_t seed, uint8_t* s1, uint8_t* s2, int64_t* stack, uint8_t* added) {
    int64_t N = p->n, top = 0;
    memset(added, 0, (size_t)N);
    stack[top++] = seed;
    added[seed] = 1;
    while (top) {
        int64_t ind = stack[--top];
        s1[ind] = !s1[ind];
        s2[ind] = !s2[ind];
        if (p->sparse) {
            for (int64_t a = p->row[ind]; a < p->row[ind + 1]; a++) {
                int64_t d = p->col[a];
                if (s1[d] != s2[d] && !added[d]) { added[d] = 1; stack[top++] = d; }
            }
        } else {
            const double* r = p->w + ind * N;
            for (int64_t i = 0; i < N; i++)
                if (fabs(r[i]) > 1e-10 && s1[i] != s2[i] && !added[i]) { stack[top++] = i; added[i] = 1; }
        }
    }
}

/* xor_icm's overlap (src/icm.cc:8-31) without the seed draw: s1 is negated
 * when more than N/2 sites differ, as there; the differing sites, ascending,
 * go to `sites`; returns their count. */
int64_t orc_overlap(const orc_problem* p, uint8_t* s1, const uint8_t* s2, int64_t* sites) {
    uint64_t N = (uint64_t)p->n, cnt = 0;
    for (uint64_t j = 0; j < N; j++) if (s1[j] ^ s2[j]) sites[cnt++] = (int64_t)j;
    if (cnt > N / 2) {
        cnt = 0;
        for (uint64_t j = 0; j < N; j++) {
            s1[j] = !s1[j];
            if (s1[j] != s2[j]) sites[cnt++] = (int64_t)j;
        }
    }
    return (int64_t)cnt;
}

/* bfs_icm (src/icm.cc:37-72) on caller states from a caller seed. */
void orc_bfs_icm(const orc_problem* p, int64_t seed, uint8_t* s1, uint8_t* s2) {
    int64_t* stack = (int64_t*)malloc(((size_t)p->n + 1) * sizeof(int64_t));
    uint8_t* added = (uint8_t*)malloc((size_t)p->n + 1);
    bfs_icm(p, seed, s1, s2, stack, added);
    free(stack);
    free(added);
}

/* icm (src/icm.cc:74-215), both replicas on rank 0. */
static int icm_step(pt_t* w, uint64_t target, uint8_t* t1, uint8_t* t2, int64_t* tmp, uint8_t* added) {
    uint64_t N = w->N;
    double beta_val = w->beta_values[target];
    int64_t a = get_replica(w, beta_val, 0), b = get_replica(w, beta_val, 1);
    if (a < 0 || b < 0) return -1;
    memcpy(t1, w->s + (uint64_t)a * N, N);
    memcpy(t2, w->s + (uint64_t)b * N, N);
    int64_t seed = xor_icm(w, t1, t2, tmp);
    if (w->tr) vpush(&w->tr->icm, &seed);
    if (seed != -1) bfs_icm(w->p, seed, t1, t2, tmp, added);
    memcpy(w->s + (uint64_t)a * N, t1, N);
    w->E[a] = orc_calculate_dE(w->p, t1, w->dE + (uint64_t)a * N);
    memcpy(w->s + (uint64_t)b * N, t2, N);
    w->E[b] = orc_calculate_dE(w->p, t2, w->dE + (uint64_t)b * N);
    return 0;
}

static uint64_t walk_ladder(const double* logdos, uint64_t nb, double min_emin, double estep,
                            double beta_start, double beta_end, double step_size, double r,
                            uint64_t num_temps, double* bv);

static double mono_seconds(void) {
    struct timespec ts;
    clock_gettime(CLOCK_MONOTONIC, &ts);
    return (double)ts.tv_sec + 1e-9 * (double)ts.tv_nsec;
}

static int solve_impl(orc_problem* p, const orc_params* prm, orc_result* res, uint8_t* best_state,
                      uint8_t* replica_states, double* final_energy, orc_trace* trace, uint64_t timed_from,
                      double* timed_s);

int orc_solve(orc_problem* p, const orc_params* prm, orc_result* res,
              uint8_t* best_state, uint8_t* replica_states, double* final_energy, orc_trace* trace) {
    return solve_impl(p, prm, res, best_state, replica_states, final_energy, trace, UINT64_MAX, NULL);
}

int orc_solve_timed(orc_problem* p, const orc_params* prm, orc_result* res, uint64_t timed_from, double* timed_s) {
    return solve_impl(p, prm, res, NULL, NULL, NULL, NULL, timed_from, timed_s);
}

static int solve_impl(orc_problem* p, const orc_params* prm, orc_result* res, uint8_t* best_state,
                      uint8_t* replica_states, double* final_energy, orc_trace* trace, uint64_t timed_from,
                      double* timed_s) {
    memset(res, 0, sizeof(*res));
    pt_t W;
    memset(&W, 0, sizeof(W));
    pt_t* w = &W;
    w->p = p;
    /* the decision trace (uniforms, exchanges, seeds) unless only the slot
     * energies are wanted */
    orc_trace* energy_tr = trace;
    if (trace && trace->energy_only) trace = NULL;
    w->tr = trace;
    w->N = (uint64_t)p->n;
    uint64_t Nt0 = prm->Nt;
    if (Nt0 < 2 || 2 * Nt0 > 2048) return -2;
    w->beta_values = (double*)calloc(2 * Nt0, sizeof(double));
    /* initialize_temperatures (src/initialization.cc:103-191) */
    if (prm->preprocess) {
        w->Nt = orc_get_beta(p, prm->T0, prm->T1, prm->inverse, Nt0, 2.0, prm->pre_step, 0.4,
                             prm->pre_samples, prm->pilot_burn_in, w->beta_values, NULL, NULL, NULL);
    } else {
        orc_beta_linspace(w->beta_values, prm->T0, prm->T1, Nt0, prm->inverse);
        w->Nt = Nt0;
    }
    uint64_t Nt = w->Nt;
    uint32_t Nc = 0;
    for (int64_t i = (int64_t)Nt - 1; i >= 0; i--) {
        if (w->beta_values[i] < p->char_scale) break;
        Nc++;
    }
    memcpy(w->beta_values + Nt, w->beta_values, Nt * sizeof(double));
    uint64_t R = 2 * Nt, N = w->N;
    w->R = R;
    w->rep_beta = (double*)malloc(R * sizeof(double));
    w->chain = (uint8_t*)malloc(R);
    for (uint64_t i = 0; i < R; i++) { w->rep_beta[i] = w->beta_values[i]; w->chain[i] = i >= Nt; }
    /* initialize_replicas (src/initialization.cc:63-76) */
    w->s = (uint8_t*)malloc(R * N);
    w->dE = (double*)malloc(R * N * sizeof(double));
    w->E = (double*)malloc(R * sizeof(double));
    w->Eg = (double*)calloc(R, sizeof(double));
    w->flips = (uint32_t*)calloc(R, sizeof(uint32_t));
    w->bestE = (double*)malloc(R * sizeof(double));
    w->bestSweep = (uint64_t*)calloc(R, sizeof(uint64_t));
    w->bestS = (uint8_t*)malloc(R * N);
    w->sweepCtr = (uint64_t*)calloc(R, sizeof(uint64_t));
    for (uint64_t i = 0; i < R; i++) {
        uint8_t* si = w->s + i * N;
        for (uint64_t j = 0; j < N; j++) si[j] = (uint8_t)orc_bernoulli_half(&p->rng);
        if (trace) for (uint64_t j = 0; j < N; j++) vpush(&trace->init, &si[j]);
        w->E[i] = orc_calculate_dE(p, si, w->dE + i * N);
        w->bestE[i] = DBL_MAX;
        memcpy(w->bestS + i * N, si, N);
    }
    /* initialize_replica_exchanges (src/initialization.cc:77-100) */
    w->order1 = (uint32_t*)malloc((Nt - 1 ? Nt - 1 : 1) * sizeof(uint32_t));
    w->order2 = (uint32_t*)malloc((Nt - 1 ? Nt - 1 : 1) * sizeof(uint32_t));
    w->bidx = (uint32_t*)malloc(R * sizeof(uint32_t));
    w->att = (uint32_t*)calloc(R, sizeof(uint32_t));
    w->succ = (uint32_t*)calloc(R, sizeof(uint32_t));
    for (uint64_t i = 0; i + 1 < Nt; i++) { w->order1[i] = (uint32_t)i; w->order2[i] = (uint32_t)i; }
    for (uint64_t i = 0; i < R; i++) w->bidx[i] = (uint32_t)i;
    w->xi = 0;
    orc_shuffle_u32(w->order1, Nt - 1, &p->rng);
    orc_shuffle_u32(w->order2, Nt - 1, &p->rng);

    uint8_t* t1 = (uint8_t*)malloc(N);
    uint8_t* t2 = (uint8_t*)malloc(N);
    uint8_t* added = (uint8_t*)malloc(N);
    int64_t* tmp = (int64_t*)malloc((N + 1) * sizeof(int64_t));
    uint64_t zero = 0;
    if (trace) vpush(&trace->off, &zero);
    int rc = 0;
    /* MAIN MCMC LOOP (src/solver.cc:67-127) */
    double t_from = 0.0;
    for (uint64_t it = 0; it < prm->pts && !rc; it++) {
        if (it == timed_from) t_from = mono_seconds();
        for (uint64_t sw = 0; sw < prm->sweeps; sw++) {
            for (uint64_t r = 0; r < R; r++) {
                uint64_t flips, used = 0;
                double* tu = NULL;
                uint64_t cap = 0;
                if (trace) {
                    /* reserve room for up to N uniforms of this sweep */
                    while (trace->u.cap < trace->u.n + N) {
                        trace->u.cap = trace->u.cap ? trace->u.cap * 2 : 1024;
                        trace->u.p = realloc(trace->u.p, trace->u.cap * trace->u.el);
                    }
                    tu = (double*)trace->u.p + trace->u.n;
                    cap = N;
                }
                flips = orc_sweep(p, w->rep_beta[r], w->s + r * N, w->dE + r * N, &w->E[r],
                                  &w->bestE[r], &w->bestSweep[r], w->bestS + r * N, w->sweepCtr[r],
                                  tu, cap, &used);
                w->flips[r] += (uint32_t)flips;
                w->sweepCtr[r]++;
                w->Eg[r] = w->E[r];
                if (trace) { trace->u.n += used; uint64_t o = trace->u.n; vpush(&trace->off, &o); }
            }
        }
        if (energy_tr) for (uint64_t k = 0; k < R; k++) vpush(&energy_tr->energy, &w->Eg[w->bidx[k]]);
        for (uint64_t m = 0; m + 1 < Nt; m++) { try_exchange(w, 0); try_exchange(w, 1); }
        if (prm->icm) {
            for (int64_t k = (int64_t)Nt - 1; k >= (int64_t)Nt - (int64_t)Nc; k--)
                if (icm_step(w, (uint64_t)k, t1, t2, tmp, added)) { rc = -3; break; }
        }
    }
    if (timed_s) *timed_s = timed_from < prm->pts ? mono_seconds() - t_from : 0.0;
    /* gather_best_energy_values (src/mpi_utils.cc:103-163), one rank */
    double best = DBL_MAX;
    uint64_t bsweep = 0;
    int64_t bi = -1;
    for (uint64_t r = 0; r < R; r++)
        if (w->bestE[r] < best) { best = w->bestE[r]; bi = (int64_t)r; bsweep = w->bestSweep[r]; }
    /* get_flips (src/mpi_utils.cc:167-176): the accumulator is an int */
    int32_t acc = 0;
    uint64_t total = 0;
    for (uint64_t r = 0; r < R; r++) { acc = (int32_t)(uint32_t)((uint64_t)(int64_t)acc + (uint64_t)w->flips[r]); total += w->flips[r]; }
    res->Nt = Nt;
    res->Nc = Nc;
    memcpy(res->beta, w->beta_values, R * sizeof(double));
    memcpy(res->swap_attempts, w->att, R * sizeof(uint32_t));
    memcpy(res->swap_successes, w->succ, R * sizeof(uint32_t));
    res->swaps = w->swaps;
    res->best_energy = best;
    res->best_sweep = bsweep;
    res->flips = (uint64_t)(int64_t)acc;
    res->flips_u64 = total;
    res->char_scale = p->char_scale;
    if (bi >= 0) {
        const uint8_t* bs = w->bestS + (uint64_t)bi * N;
        res->best_state_energy = orc_energy(p, bs);
        res->best_maxcut = orc_maxcut(p, bs);
        if (best_state) memcpy(best_state, bs, N);
    } else if (!rc) {
        rc = -4; /* no replica ever accepted a flip: the reference has no best state */
    }
    if (replica_states) memcpy(replica_states, w->s, R * N);
    if (final_energy) memcpy(final_energy, w->E, R * sizeof(double));
    free(t1); free(t2); free(added); free(tmp);
    free(w->beta_values); free(w->rep_beta); free(w->chain); free(w->s); free(w->dE); free(w->E); free(w->Eg);
    free(w->flips); free(w->bestE); free(w->bestSweep); free(w->bestS); free(w->sweepCtr);
    free(w->order1); free(w->order2); free(w->bidx); free(w->att); free(w->succ);
    return rc;
}

/* ========================================================= Multihistogram */
static inline uint64_t to_bin(double e, double emin, double estep) {   /* :11-13 */
    return (uint64_t)floor((e - emin) / estep);
}

static inline double logplusexp(double x1, double l2) {                 /* :20-27 */
    double l1 = log(x1);
    if (l1 < l2) { double t = l1; l1 = l2; l2 = t; }
    double x = exp(l2 - l1);
    return l1 + log1p(x);
}

double orc_logplusexp2(double l1, double l2) {
    if (l1 < l2) { double t = l1; l1 = l2; l2 = t; }
    double x = exp(l2 - l1);
    return l1 + log1p(x);
}

double orc_partition_func(const double* logdos, uint64_t nb, double beta, double emin, double estep) {
    double logz = 1;
    int first = 1;
    for (uint64_t i = 0; i < nb; i++) {
        double e = (double)i * estep + emin;
        double logboltz = -beta * e;
        if (first) { first = 0; logz = logboltz + logdos[i]; }
        else logz = orc_logplusexp2(logz, logboltz + logdos[i]);
    }
    return logz;
}

uint64_t orc_calculate_dos(const uint32_t* hist, const uint64_t* hist_off, const uint64_t* hist_len,
                           uint64_t nt, const double* pf, const double* emin_values,
                           const double* beta_hist, double estep, double min_emin, double max_emax,
                           uint64_t n, double* logdos) {
    uint64_t nbins = (uint64_t)ceil((max_emax - min_emin) / estep);
    double logn = log((double)n);
    double e = min_emin;
    for (uint64_t i = 0; i < nbins; i++, e += estep) {
        double lognum = 1, logdenom = 1;
        int firstnum = 1, firstdenom = 1;
        for (uint64_t j = 0; j < nt; j++) {
            double term = logn - pf[j] - beta_hist[j] * e;
            if (firstdenom) { firstdenom = 0; logdenom = term; }
            else logdenom = orc_logplusexp2(term, logdenom);
            double emin_j = emin_values[j];
            if (e < emin_j) continue;
            double index = (double)to_bin(e, emin_j, estep);
            if (index >= (double)hist_len[j]) continue;
            uint32_t hv = hist[hist_off[j] + (uint64_t)index];
            if (firstnum && hv) { firstnum = 0; lognum = log((double)hv); }
            else if (!firstnum && hv) lognum = logplusexp((double)hv, lognum);
        }
        logdos[i] = firstnum ? -DBL_MAX : lognum - logdenom;
    }
    return nbins;
}

uint64_t orc_partition_iterate(const uint32_t* hist, const uint64_t* hist_off, const uint64_t* hist_len,
                               uint64_t nt, const double* beta_hist, const double* emin_values,
                               double estep, uint64_t n, double max_emax, double* logdos, double* pf) {
    double emin = emin_values[0];
    for (uint64_t i = 1; i < nt; i++) if (emin_values[i] < emin) emin = emin_values[i];
    for (uint64_t i = 0; i < nt; i++) pf[i] = 0;
    uint64_t iters = 0;
    double max_diff;
    do {
        max_diff = 0;
        uint64_t nb = orc_calculate_dos(hist, hist_off, hist_len, nt, pf, emin_values, beta_hist,
                                        estep, emin, max_emax, n, logdos);
        for (uint64_t i = 0; i < nt; i++) {
            double tz = orc_partition_func(logdos, nb, beta_hist[i], emin, estep);
            max_diff += pow(fabs(pf[i] - tz) / fabs(tz), 2.0);
            pf[i] = tz;
        }
        iters++;
    } while (max_diff > 1e-7);
    return iters;
}

static void get_pe_vec(const double* logdos, uint64_t nb, double* logpE, double emin, double beta,
                       double logpartition, double estep) {                                 /* :255-260 */
    double e = emin;
    for (uint64_t i = 0; i < nb; i++, e += estep) logpE[i] = logdos[i] - e * beta - logpartition;
}

double orc_acceptance_rate(const double* logdos, uint64_t nb, const double* p1, const double* p2,
                           double beta_1, double beta_2, double estep, double emin) {
    (void)logdos;
    double r = 1, p1i, p12, e1, e2 = 0;
    int first = 1;
    e1 = emin;
    for (uint64_t i = 0; i < nb; i++, e1 += estep) {
        p1i = p1[i];
        for (uint64_t j = 0; j <= i; j++) {
            if (first) { first = 0; r = p1i + p2[j]; }
            else r = orc_logplusexp2(r, p1i + p2[j]);
        }
        e2 = e1 + estep;
        for (uint64_t j = i + 1; j < nb; j++, e2 += estep) {
            p12 = (beta_1 - beta_2) * (e1 - e2);
            if (first) { first = 0; r = p1i + p2[j] + p12; }
            else r = orc_logplusexp2(r, p1i + p2[j] + p12);
        }
    }
    return exp(r);
}

static uint64_t walk_ladder(const double* logdos, uint64_t nb, double min_emin, double estep,
                            double beta_start, double beta_end, double step_size, double r,
                            uint64_t num_temps, double* bv) {
    bv[0] = beta_start;
    double partition_last = orc_partition_func(logdos, nb, beta_start, min_emin, estep);
    double step = step_size;
    double* prev = (double*)malloc((nb ? nb : 1) * sizeof(double));
    double* curr = (double*)malloc((nb ? nb : 1) * sizeof(double));
    get_pe_vec(logdos, nb, prev, min_emin, beta_start, partition_last, estep);
    uint64_t i;
    for (i = 1; i < num_temps; i++) {
        double beta_prev = bv[i - 1];
        bv[i] = beta_prev;
        double partition_curr = 0, r_curr = 0, r_last = -1;
        int cont;
        for (;;) {
            cont = 0;
            double beta_orig = bv[i];
            bv[i] = 1 / (1 / bv[i] + step);
            partition_curr = orc_partition_func(logdos, nb, bv[i], min_emin, estep);
            get_pe_vec(logdos, nb, curr, min_emin, bv[i], partition_curr, estep);
            r_curr = orc_acceptance_rate(logdos, nb, prev, curr, beta_prev, bv[i], estep, min_emin);
            if ((r - r_curr) > 0.05) {
                bv[i] = beta_orig;
                step /= 2;
                cont = 1;
            } else if (r_last > 0 && fabs(r_curr - r_last) < 5e-2) {
                step *= 2;
            } else {
                r_last = r_curr;
            }
            if (!((r_curr > r && bv[i] > beta_end) || cont)) break;
        }
        if (bv[i] <= beta_end) break;
        partition_last = partition_curr;
        memcpy(prev, curr, nb * sizeof(double));
    }
    free(prev);
    free(curr);
    return i;
}

uint64_t orc_cae_walk(const double* logdos, uint64_t nb, double min_emin, double estep,
                      double beta_start, double beta_end, double step_size, double r,
                      uint64_t num_temps, double* beta_out) {
    return walk_ladder(logdos, nb, min_emin, estep, beta_start, beta_end, step_size, r, num_temps, beta_out);
}

/* The pilot run of gather_samples (:76-151) on hist_betas hb[0..Nt) and the
 * per-temperature histograms of make_histogram (:45-69).  Returns a malloc'd
 * concatenation of the histograms (row j at hoff[j], length hlen[j]); emin_v,
 * emaxv receive each row's energy range and *n_out the int-accumulated count
 * of row 0 (src/cae_estimator.cc:343). */
static uint32_t* pilot_histograms(orc_problem* p, const double* hb, uint64_t Nt, double estep,
                                  uint64_t num_samples, uint64_t burn_in, uint64_t* hoff, uint64_t* hlen,
                                  double* emin_v, double* emaxv, uint64_t* n_out);

/* gather_samples (:76-151) + make_histogram (:45-69) + get_beta (:295-428) */
uint64_t orc_get_beta(orc_problem* p, double T0, double T1, int inverse, uint64_t num_temps,
                      double estep, double step_size, double r, uint64_t num_samples,
                      uint64_t burn_in, double* beta_out,
                      double* hist_betas_out, double* emin_out, double* emax_out) {
    uint64_t Nt = num_temps;
    double beta_start, beta_end;
    if (inverse) { beta_start = T0; beta_end = T1; }
    else { beta_start = 1 / T0; beta_end = 1 / T1; }
    if (beta_start < beta_end) { double t = beta_start; beta_start = beta_end; beta_end = t; }
    double beta_step = (beta_end - beta_start) / (double)(Nt - 1);
    double* hb = (double*)malloc(Nt * sizeof(double));
    double beta = beta_start;
    for (uint64_t i = 0; i < Nt; i++, beta += beta_step) hb[i] = beta;
    uint64_t* hoff = (uint64_t*)malloc(Nt * sizeof(uint64_t));
    uint64_t* hlen = (uint64_t*)malloc(Nt * sizeof(uint64_t));
    double* emin_v = (double*)malloc(Nt * sizeof(double));
    double* emaxv = (double*)malloc(Nt * sizeof(double));
    uint64_t n = 0;
    uint32_t* hist = pilot_histograms(p, hb, Nt, estep, num_samples, burn_in, hoff, hlen, emin_v, emaxv, &n);
    double max_emax = -DBL_MAX, min_emin = DBL_MAX;
    for (uint64_t i = 0; i < Nt; i++) {
        if (emaxv[i] > max_emax) max_emax = emaxv[i];
        if (emin_v[i] < min_emin) min_emin = emin_v[i];
    }
    uint64_t nb = (uint64_t)ceil((max_emax - min_emin) / estep);
    double* logdos = (double*)malloc((nb ? nb : 1) * sizeof(double));
    double* pf = (double*)malloc(Nt * sizeof(double));
    orc_partition_iterate(hist, hoff, hlen, Nt, hb, emin_v, estep, n, max_emax, logdos, pf);
    uint64_t cnt = walk_ladder(logdos, nb, min_emin, estep, beta_start, beta_end, step_size, r, Nt, beta_out);
    if (hist_betas_out) memcpy(hist_betas_out, hb, Nt * sizeof(double));
    if (emin_out) memcpy(emin_out, emin_v, Nt * sizeof(double));
    if (emax_out) memcpy(emax_out, emaxv, Nt * sizeof(double));
    free(hb); free(hoff); free(hlen); free(emin_v); free(emaxv); free(hist); free(logdos); free(pf);
    return cnt;
}

uint64_t orc_pilot(orc_problem* p, const double* hb, uint64_t Nt, double estep, uint64_t num_samples,
                   uint64_t burn_in, uint32_t* hist_out, uint64_t hist_cap, uint64_t* hoff, uint64_t* hlen,
                   double* emin_v, double* emaxv, uint64_t* n_out) {
    uint32_t* h = pilot_histograms(p, hb, Nt, estep, num_samples, burn_in, hoff, hlen, emin_v, emaxv, n_out);
    uint64_t tot = hoff[Nt - 1] + hlen[Nt - 1];
    if (hist_out) memcpy(hist_out, h, (tot < hist_cap ? tot : hist_cap) * sizeof(uint32_t));
    free(h);
    return tot;
}

static uint32_t* pilot_histograms(orc_problem* p, const double* hb, uint64_t Nt, double estep,
                                  uint64_t num_samples, uint64_t burn_in, uint64_t* hoff, uint64_t* hlen,
                                  double* emin_v, double* emaxv, uint64_t* n_out) {
    uint64_t N = (uint64_t)p->n;
    /* pilot run */
    uint8_t* s = (uint8_t*)malloc(Nt * N);
    double* dE = (double*)malloc(Nt * N * sizeof(double));
    double* E = (double*)malloc(Nt * sizeof(double));
    double* rb = (double*)malloc(Nt * sizeof(double));
    double* bE = (double*)malloc(Nt * sizeof(double));
    uint64_t* bS = (uint64_t*)calloc(Nt, sizeof(uint64_t));
    uint64_t* ctr = (uint64_t*)calloc(Nt, sizeof(uint64_t));
    uint32_t* order = (uint32_t*)malloc((Nt ? Nt : 1) * sizeof(uint32_t));
    uint32_t* ri = (uint32_t*)malloc(Nt * sizeof(uint32_t));
    double* logs = (double*)malloc((Nt * (num_samples ? num_samples : 1)) * sizeof(double));
    for (uint64_t ind = 0; ind < Nt; ind++) {
        ri[ind] = (uint32_t)ind;
        if (ind + 1 < Nt) order[ind] = (uint32_t)ind;
        for (uint64_t i = 0; i < N; i++) s[ind * N + i] = (uint8_t)orc_bernoulli_half(&p->rng);
        E[ind] = orc_calculate_dE(p, s + ind * N, dE + ind * N);
        rb[ind] = hb[ind];
        bE[ind] = DBL_MAX;
    }
    for (uint64_t it = 0; it < burn_in + num_samples; it++) {
        for (uint64_t rind = 0; rind < Nt; rind++) {
            uint32_t q = ri[rind];
            orc_sweep(p, rb[q], s + q * N, dE + q * N, &E[q], &bE[q], &bS[q], NULL, ctr[q], NULL, 0, NULL);
            ctr[q]++;
            if (it >= burn_in) logs[rind * num_samples + (it - burn_in)] = E[q];
        }
        orc_shuffle_u32(order, Nt - 1, &p->rng);
        for (uint64_t a = 0; a + 1 < Nt; a++) {
            uint32_t index = order[a];
            uint32_t q1 = ri[index], q2 = ri[index + 1];
            double e1 = E[q1], e2 = E[q2];
            double b1 = hb[index], b2 = hb[index + 1];
            double logboltz = (e1 - e2) * (b1 - b2);
            double rng = orc_canonical(&p->rng);
            if (log(rng) < logboltz) {
                ri[index] = q2; ri[index + 1] = q1;
                rb[q1] = b2; rb[q2] = b1;
            }
        }
    }
    /* histograms per temperature slot */
    uint64_t tot = 0;
    for (uint64_t i = 0; i < Nt; i++) {
        double* lg = logs + i * num_samples;
        double mn = lg[0], mx = lg[0];
        for (uint64_t k = 1; k < num_samples; k++) { if (lg[k] < mn) mn = lg[k]; if (lg[k] > mx) mx = lg[k]; }
        emin_v[i] = mn; emaxv[i] = mx;
        hlen[i] = (uint64_t)ceil((mx - mn) / estep) + 1;
        hoff[i] = tot;
        tot += hlen[i];
    }
    uint32_t* hist = (uint32_t*)calloc(tot ? tot : 1, sizeof(uint32_t));
    for (uint64_t i = 0; i < Nt; i++) {
        double* lg = logs + i * num_samples;
        for (uint64_t k = 0; k < num_samples; k++) hist[hoff[i] + to_bin(lg[k], emin_v[i], estep)]++;
    }
    /* n = accumulate(histograms[0]) with an int accumulator */
    int32_t nacc = 0;
    for (uint64_t b = 0; b < hlen[0]; b++) nacc = (int32_t)(nacc + (int32_t)hist[hoff[0] + b]);
    *n_out = (uint64_t)(int64_t)nacc;
    free(s); free(dE); free(E); free(rb); free(bE); free(bS); free(ctr); free(order); free(ri); free(logs);
    return hist;
}
