/*
 * gbca_oracle.c — CPU oracle (test infrastructure only; never linked into the
 * product). A restatement in C of the per-cell arithmetic of
 * CellularAutomataCore.jl's ReferenceBackend and ArrayBackend for Int8
 * Life-like / Larger-than-Life / Generations / forest-fire rules and for Lenia.
 * Compile with -ffp-contract=off: Julia does not fuse `s += w * x`.
 */
#include "gbca_oracle.h"

#include <math.h>
#include <pthread.h>
#include <stdlib.h>
#include <string.h>

/* ------------------------------------------------------------ Philox (random.jl) */

#define OR_M0 0xD2511F53u
#define OR_M1 0xCD9E8D57u
#define OR_W0 0x9E3779B9u
#define OR_W1 0xBB67AE85u

/* random.jl:24-37: ten rounds; the key is bumped after rounds 1..9. */
void or_philox4x32(const uint32_t ctr[4], const uint32_t key[2], uint32_t out[4]) {
    uint32_t c0 = ctr[0], c1 = ctr[1], c2 = ctr[2], c3 = ctr[3];
    uint32_t k0 = key[0], k1 = key[1];
    for (int round = 1; round <= 10; ++round) {
        uint64_t p0 = (uint64_t)OR_M0 * (uint64_t)c0;
        uint64_t p1 = (uint64_t)OR_M1 * (uint64_t)c2;
        uint32_t hi0 = (uint32_t)(p0 >> 32), lo0 = (uint32_t)p0;
        uint32_t hi1 = (uint32_t)(p1 >> 32), lo1 = (uint32_t)p1;
        uint32_t n0 = hi1 ^ c1 ^ k0, n1 = lo1, n2 = hi0 ^ c3 ^ k1, n3 = lo0;
        c0 = n0; c1 = n1; c2 = n2; c3 = n3;
        if (round < 10) { k0 += OR_W0; k1 += OR_W1; }
    }
    out[0] = c0; out[1] = c1; out[2] = c2; out[3] = c3;
}

/* random.jl:102-107: ctr = (id lo, id hi, t mod 2^32, k), key = (seed lo, seed hi). */
static void or_draw(uint64_t seed, uint64_t id, int64_t t, uint32_t k, uint32_t r[4]) {
    uint32_t ctr[4] = {(uint32_t)id, (uint32_t)(id >> 32), (uint32_t)(uint64_t)t, k};
    uint32_t key[2] = {(uint32_t)seed, (uint32_t)(seed >> 32)};
    or_philox4x32(ctr, key, r);
}

/* random.jl:116-120 */
double or_uniform(uint64_t seed, uint64_t cellid, int64_t t, uint32_t k) {
    uint32_t r[4];
    or_draw(seed, cellid, t, k, r);
    uint64_t bits = ((uint64_t)r[0] << 32) | (uint64_t)r[1];
    return (double)(bits >> 11) * 0x1.0p-53;
}

/* random.jl:109-114 */
float or_uniform32(uint64_t seed, uint64_t cellid, int64_t t, uint32_t k) {
    uint32_t r[4];
    or_draw(seed, cellid, t, k, r);
    return (float)(r[0] >> 8) * (1.0f / 16777216.0f);
}

/* random.jl:129-130: bernoulli = uniform < p, in the precision of p. */
static int or_bernoulli(uint64_t seed, uint64_t id, int64_t t, uint32_t k, double p, int f32) {
    if (f32) return or_uniform32(seed, id, t, k) < (float)p;
    return or_uniform(seed, id, t, k) < p;
}

/* ------------------------------------------------------ neighbourhoods, boundaries */

/* neighbourhoods.jl:124-153: CartesianIndices((-r:r, -r:r)), first axis fastest. */
int or_offsets(int32_t nbhd, int32_t radius, int32_t* off) {
    int m = 0;
    for (int dj = -radius; dj <= radius; ++dj)
        for (int di = -radius; di <= radius; ++di) {
            if (di == 0 && dj == 0) continue;
            if (nbhd == OR_VON_NEUMANN && abs(di) + abs(dj) > radius) continue;
            off[2 * m] = di;
            off[2 * m + 1] = dj;
            ++m;
        }
    return m;
}

static int64_t or_mod(int64_t a, int64_t n) {
    int64_t m = a % n;
    return m < 0 ? m + n : m;
}

/* spaces.jl:46-51. Returns the mapped 1-based index; *outside only for Constant. */
static int64_t or_map_axis(int32_t b, int64_t j, int64_t n, int* outside) {
    *outside = 0;
    if (b == OR_PERIODIC) return or_mod(j - 1, n) + 1;
    if (b == OR_REFLECTING) {
        int64_t m = or_mod(j - 1, 2 * n);
        return m < n ? m + 1 : 2 * n - m;
    }
    *outside = !(1 <= j && j <= n);
    return j;
}

/* backends.jl:177-184 + :196-200: the value read at unpadded (i, j); beyond
 * several Constant edges the highest-numbered axis wins. */
static int8_t or_boundary_read(const or_problem* P, const int8_t* u, int64_t i, int64_t j) {
    int o1, o2;
    int64_t a = or_map_axis(P->boundary[0], i, P->n1, &o1);
    int64_t b = or_map_axis(P->boundary[1], j, P->n2, &o2);
    if (o2) return (int8_t)P->constant[1];
    if (o1) return (int8_t)P->constant[0];
    return u[(a - 1) + (b - 1) * P->n1];
}

/* ------------------------------------------------------------------ rules */

/* rules.jl:377-389 (Life), :446-456 (Generations); forest fire from the
 * package README (LocalRule on Int8 codes 0 empty, 1 tree, 2 fire). */
static int8_t or_rule(const or_problem* P, int8_t c, const int8_t* nb, int m, uint64_t id,
                      int64_t t, const double* params) {
    if (P->rule == OR_RULE_FOREST_FIRE) {
        if (c == 2) return 0;
        if (c == 0) return or_bernoulli(P->seed, id, t, 1, params[0], P->params_f32) ? 1 : 0;
        for (int k = 0; k < m; ++k)
            if (nb[k] == 2) return 2;
        return or_bernoulli(P->seed, id, t, 2, params[1], P->params_f32) ? 2 : 1;
    }
    int n = 0;
    for (int k = 0; k < m; ++k) n += (nb[k] == 1);
    if (P->rule == OR_RULE_LIFE) {
        uint64_t mask = c == 1 ? P->survive : P->birth;
        return (int8_t)(n < 64 ? (mask >> n) & 1u : 0u);
    }
    /* Generations */
    int s = c;
    if (s == 0) return (int8_t)(n < 64 ? (P->birth >> n) & 1u : 0u);
    if (s == 1) {
        if (n < 64 && ((P->survive >> n) & 1u)) return c;
        return (int8_t)(P->states > 2 ? 2 : 0);
    }
    return (int8_t)(s + 1 < P->states ? s + 1 : 0);
}

/* schemes.jl:84-93 */
static int or_gate_open(const or_problem* P, int gate, int64_t i, int64_t j, uint64_t id, int64_t t) {
    if (P->scheme == OR_STOCHASTIC) {
        if (P->scheme_p_f32) return or_uniform32(P->seed, id, t, 0) < (float)P->scheme_p;
        return or_uniform(P->seed, id, t, 0) < P->scheme_p;
    }
    if (P->scheme == OR_CHECKERBOARD) return ((i + j) & 1) == (gate == 1);
    return 1;
}

static int or_ngates(const or_problem* P) { return P->scheme == OR_CHECKERBOARD ? 2 : 1; }

/* ------------------------------------------------------------ environment */

/* Julia's promotion for a product: Float32 * Float32 stays Float32, else Float64. */
typedef struct { int f32; float f; double d; } or_num;

static or_num or_num32(float f) { or_num r; r.f32 = 1; r.f = f; r.d = (double)f; return r; }
static or_num or_num64(double d) { or_num r; r.f32 = 0; r.f = (float)d; r.d = d; return r; }
static or_num or_mul(or_num a, or_num b) {
    if (a.f32 && b.f32) return or_num32(a.f * b.f);
    return or_num64(a.d * b.d);
}

/* environment.jl:151-160: field values of every cell from the state, boundary
 * semantics on every read, taps in order. Columns j0..j1 (1-based). */
typedef struct {
    const or_problem* P;
    const or_env* E;
    const int8_t* cur;
    double* f64;
    float* f32;
    const float* w32;
    int64_t j0, j1;
} or_field_job;

static void* or_field_worker(void* arg) {
    or_field_job* J = (or_field_job*)arg;
    const or_problem* P = J->P;
    const or_env* E = J->E;
    for (int64_t j = J->j0; j <= J->j1; ++j)
        for (int64_t i = 1; i <= P->n1; ++i) {
            double s = 0.0;
            float sf = 0.0f;
            for (int k = 0; k < E->ntaps; ++k) {
                int8_t v = or_boundary_read(P, J->cur, i + E->taps[2 * k], j + E->taps[2 * k + 1]);
                double x = E->source ? (double)v : (v == 1 ? 1.0 : 0.0);
                if (E->field_f32) sf += J->w32[k] * (float)x;
                else s += E->weights[k] * x;
            }
            int64_t lin = (i - 1) + (j - 1) * P->n1;
            if (E->field_f32) J->f32[lin] = sf;
            else J->f64[lin] = s;
        }
    return NULL;
}

static void or_compute_field(const or_problem* P, const or_env* E, const int8_t* cur, double* f64, float* f32,
                             int nthreads) {
    float* w32 = (float*)malloc(sizeof(float) * (size_t)E->ntaps);
    for (int k = 0; k < E->ntaps; ++k) w32[k] = (float)E->weights[k];
    int nt = nthreads > 1 ? nthreads : 1;
    if (nt > 64) nt = 64;
    if (nt > P->n2) nt = (int)P->n2;
    or_field_job jobs[64];
    pthread_t th[64];
    for (int k = 0; k < nt; ++k) {
        or_field_job* J = &jobs[k];
        J->P = P; J->E = E; J->cur = cur; J->f64 = f64; J->f32 = f32; J->w32 = w32;
        J->j0 = (k * P->n2) / nt + 1;
        J->j1 = ((k + 1) * P->n2) / nt;
    }
    if (nt == 1) or_field_worker(&jobs[0]);
    else {
        for (int k = 0; k < nt; ++k) pthread_create(&th[k], NULL, or_field_worker, &jobs[k]);
        for (int k = 0; k < nt; ++k) pthread_join(th[k], NULL);
    }
    free(w32);
}

int or_kernel_field(const or_problem* P, const or_env* E, const int8_t* u, double* f64, float* f32) {
    if (!E || E->ntaps < 1) return -3;
    or_compute_field(P, E, u, f64, f32, 1);
    return 0;
}

/* The typed kernel-field SI rule (test/backend_conformance.jl:52-57,72-75). */
static int8_t or_si_rule(const or_problem* P, const or_env* E, int8_t c, int64_t lin, uint64_t id, int64_t t,
                         const double* params, const double* f64, const float* f32) {
    if (c == 1) return c;
    or_num lam = P->params_f32 ? or_num32((float)params[0]) : or_num64(params[0]);
    if (E->cov) {
        int64_t nt = E->cov_nt > 0 ? E->cov_nt : 1;
        int64_t slice = or_mod(t, nt);                      /* mod1(t + 1, nt) - 1 */
        int64_t at = lin + slice * P->n1 * P->n2;
        lam = or_mul(lam, E->cov_f32 ? or_num32(((const float*)E->cov)[at]) : or_num64(((const double*)E->cov)[at]));
    }
    lam = or_mul(lam, E->field_f32 ? or_num32(f32[lin]) : or_num64(f64[lin]));
    if (lam.f32) {
        float e = (float)exp(-(double)lam.f);              /* Float32 exp, correctly rounded */
        float q = 1.0f - e;
        return or_uniform32(P->seed, id, t, 1) < q ? 1 : c;
    }
    double q = 1.0 - exp(-lam.d);
    return or_uniform(P->seed, id, t, 1) < q ? 1 : c;
}

static int or_masked(const or_env* E, int64_t lin) { return E && E->mask && !E->mask[lin]; }

/* ------------------------------------------------------- ReferenceBackend step */

/* backends.jl:264-278 (one gated sweep) and :314-322 (gates of one step); fields are
 * computed once per step, before the gates (backends.jl:494-506). */
int or_step_reference_env(const or_problem* P, const or_env* E, int8_t* cur, int64_t t, const double* params) {
    int32_t off[2 * 201 * 201];
    if (P->radius < 1 || P->radius > 100) return -1;
    if (P->rule == OR_RULE_SI_FIELD && (!E || E->ntaps < 1)) return -3;
    int m = or_offsets(P->nbhd, P->radius, off);
    int64_t n1 = P->n1, n2 = P->n2, n = n1 * n2;
    int8_t* next = (int8_t*)malloc((size_t)n);
    int8_t* nb = (int8_t*)malloc((size_t)m);
    double* f64 = NULL;
    float* f32 = NULL;
    if (E && E->ntaps > 0) {
        f64 = (double*)malloc(sizeof(double) * (size_t)n);
        f32 = (float*)malloc(sizeof(float) * (size_t)n);
    }
    if (!next || !nb || (E && E->ntaps > 0 && (!f64 || !f32))) { free(next); free(nb); free(f64); free(f32); return -2; }
    if (f64) or_compute_field(P, E, cur, f64, f32, 1);
    for (int g = 0; g < or_ngates(P); ++g) {
        for (int64_t j = 1; j <= n2; ++j)
            for (int64_t i = 1; i <= n1; ++i) {
                int64_t lin = (i - 1) + (j - 1) * n1;
                uint64_t id = (uint64_t)(lin + 1);
                int8_t c = cur[lin];
                if (or_masked(E, lin) || !or_gate_open(P, g, i, j, id, t)) {
                    next[lin] = c;
                    continue;
                }
                if (P->rule == OR_RULE_SI_FIELD) {
                    next[lin] = or_si_rule(P, E, c, lin, id, t, params, f64, f32);
                    continue;
                }
                for (int k = 0; k < m; ++k)
                    nb[k] = or_boundary_read(P, cur, i + off[2 * k], j + off[2 * k + 1]);
                next[lin] = or_rule(P, c, nb, m, id, t, params);
            }
        memcpy(cur, next, (size_t)n);
    }
    free(next); free(nb); free(f64); free(f32);
    return 0;
}

int or_step_reference(const or_problem* P, int8_t* cur, int64_t t, const double* params) {
    return or_step_reference_env(P, NULL, cur, t, params);
}

/* ------------------------------------------------------------ ArrayBackend run */

typedef struct {
    const or_problem* P;
    int8_t* cur;
    int8_t* next;
    int64_t h, p1, p2;       /* halo and padded dims */
    const int64_t* lin;      /* padded linear offsets of the neighbourhood */
    int m;
    int64_t t;
    int gate;
    const double* params;
    int64_t nchunks;
    int64_t next_chunk;      /* dynamic chunk counter (Threads.@threads :dynamic) */
    pthread_mutex_t lock;
    const or_env* E;
    const double* f64;       /* field values of this step (unpadded) */
    const float* f32;
} or_sweep_job;

/* backends.jl:425-442: every halo cell gets the boundary value of its unpadded index. */
static void or_fill_halo(const or_problem* P, int8_t* cur, int64_t h, int64_t p1, int64_t p2) {
    /* the interior of the padded array, viewed as an unpadded state, is read
     * through the boundary mapping; mapped indices are always interior */
    for (int64_t pj = 0; pj < p2; ++pj)
        for (int64_t pi = 0; pi < p1; ++pi) {
            int64_t i = pi - h + 1, j = pj - h + 1;
            if (i >= 1 && i <= P->n1 && j >= 1 && j <= P->n2) continue;
            int o1, o2;
            int64_t a = or_map_axis(P->boundary[0], i, P->n1, &o1);
            int64_t b = or_map_axis(P->boundary[1], j, P->n2, &o2);
            int8_t v;
            if (o2) v = (int8_t)P->constant[1];
            else if (o1) v = (int8_t)P->constant[0];
            else v = cur[(a - 1 + h) + (b - 1 + h) * p1];
            cur[pi + pj * p1] = v;
        }
}

/* backends.jl:444-455 over one slab of columns lo..hi (1-based, inclusive). */
static void or_sweep_slab(or_sweep_job* J, int64_t lo, int64_t hi) {
    const or_problem* P = J->P;
    int8_t nb[128 * 128];
    for (int64_t j = lo; j <= hi; ++j)
        for (int64_t i = 1; i <= P->n1; ++i) {
            int64_t pos = (i - 1 + J->h) + (j - 1 + J->h) * J->p1;
            uint64_t id = (uint64_t)((i - 1) + (j - 1) * P->n1 + 1);
            int8_t c = J->cur[pos];
            int64_t lin = (i - 1) + (j - 1) * P->n1;
            if (or_masked(J->E, lin) || !or_gate_open(P, J->gate, i, j, id, J->t)) {
                J->next[pos] = c;
                continue;
            }
            if (P->rule == OR_RULE_SI_FIELD) {
                J->next[pos] = or_si_rule(P, J->E, c, lin, id, J->t, J->params, J->f64, J->f32);
                continue;
            }
            for (int k = 0; k < J->m; ++k) nb[k] = J->cur[pos + J->lin[k]];
            J->next[pos] = or_rule(P, c, nb, J->m, id, J->t, J->params);
        }
}

static void* or_sweep_worker(void* arg) {
    or_sweep_job* J = (or_sweep_job*)arg;
    for (;;) {
        pthread_mutex_lock(&J->lock);
        int64_t c = J->next_chunk++;
        pthread_mutex_unlock(&J->lock);
        if (c > J->nchunks) break;
        /* backends.jl:465-466 */
        int64_t lo = ((c - 1) * J->P->n2) / J->nchunks + 1;
        int64_t hi = (c * J->P->n2) / J->nchunks;
        or_sweep_slab(J, lo, hi);
    }
    return NULL;
}

int or_run_array(const or_problem* P, int8_t* state, int64_t t0, int64_t nsteps,
                 const double* params, int32_t nthreads) {
    return or_run_array_env(P, NULL, state, t0, nsteps, params, nthreads);
}

int or_run_array_env(const or_problem* P, const or_env* E, int8_t* state, int64_t t0, int64_t nsteps,
                     const double* params, int32_t nthreads) {
    int32_t off[2 * 201 * 201];
    if (P->radius < 1 || P->radius > 63) return -1;
    if (P->rule == OR_RULE_SI_FIELD && (!E || E->ntaps < 1)) return -3;
    double* f64 = NULL;
    float* f32 = NULL;
    int8_t* flat = NULL;
    if (E && E->ntaps > 0) {
        f64 = (double*)malloc(sizeof(double) * (size_t)(P->n1 * P->n2));
        f32 = (float*)malloc(sizeof(float) * (size_t)(P->n1 * P->n2));
        flat = (int8_t*)malloc((size_t)(P->n1 * P->n2));
        if (!f64 || !f32 || !flat) { free(f64); free(f32); free(flat); return -2; }
    }
    int m = or_offsets(P->nbhd, P->radius, off);
    int64_t h = P->radius > 1 ? P->radius : 1; /* backends.jl:405 */
    int64_t p1 = P->n1 + 2 * h, p2 = P->n2 + 2 * h;
    int8_t* cur = (int8_t*)calloc((size_t)(p1 * p2), 1);
    int8_t* next = (int8_t*)calloc((size_t)(p1 * p2), 1);
    int64_t* lin = (int64_t*)malloc(sizeof(int64_t) * (size_t)m);
    pthread_t* th = (pthread_t*)malloc(sizeof(pthread_t) * (size_t)(nthreads > 1 ? nthreads : 1));
    if (!cur || !next || !lin || !th) { free(cur); free(next); free(lin); free(th); return -2; }
    for (int k = 0; k < m; ++k) lin[k] = off[2 * k] + off[2 * k + 1] * p1;
    for (int64_t j = 0; j < P->n2; ++j)
        memcpy(cur + h + (j + h) * p1, state + j * P->n1, (size_t)P->n1);
    or_sweep_job J;
    memset(&J, 0, sizeof J);
    J.P = P; J.h = h; J.p1 = p1; J.p2 = p2; J.lin = lin; J.m = m; J.params = params;
    J.E = E; J.f64 = f64; J.f32 = f32;
    pthread_mutex_init(&J.lock, NULL);
    for (int64_t s = 0; s < nsteps; ++s) {
        J.t = t0 + s;
        or_fill_halo(P, cur, h, p1, p2);
        if (f64) {  /* backends.jl:481-492: fields from the state at the start of the step */
            for (int64_t j = 0; j < P->n2; ++j)
                memcpy(flat + j * P->n1, cur + h + (j + h) * p1, (size_t)P->n1);
            or_compute_field(P, E, flat, f64, f32, nthreads);
        }
        for (int g = 0; g < or_ngates(P); ++g) {
            if (g > 0) or_fill_halo(P, cur, h, p1, p2);
            J.cur = cur; J.next = next; J.gate = g;
            if (nthreads > 1) {
                J.nchunks = P->n2 < 4 * (int64_t)nthreads ? P->n2 : 4 * (int64_t)nthreads;
                J.next_chunk = 1;
                for (int k = 0; k < nthreads; ++k) pthread_create(&th[k], NULL, or_sweep_worker, &J);
                for (int k = 0; k < nthreads; ++k) pthread_join(th[k], NULL);
            } else {
                or_sweep_slab(&J, 1, P->n2);
            }
            int8_t* tmp = cur; cur = next; next = tmp;   /* swap! backends.jl:512-515 */
        }
    }
    for (int64_t j = 0; j < P->n2; ++j)
        memcpy(state + j * P->n1, cur + h + (j + h) * p1, (size_t)P->n1);
    pthread_mutex_destroy(&J.lock);
    free(cur); free(next); free(lin); free(th);
    free(f64); free(f32); free(flat);
    return 0;
}

/* ------------------------------------------------------------------ measures */

void or_state_counts(const int8_t* u, int64_t n, int64_t* counts, int32_t nvals, int64_t* other) {
    for (int v = 0; v < nvals; ++v) counts[v] = 0;
    int64_t o = 0;
    for (int64_t k = 0; k < n; ++k) {
        int v = u[k];
        if (v >= 0 && v < nvals) counts[v]++;
        else o++;
    }
    if (other) *other = o;
}

void or_soup(uint64_t seed, int64_t n1, int64_t n2, double density, int8_t* out) {
    const float p = (float)density;
    for (int64_t q = 0; q < n1 * n2; ++q)
        out[q] = (int8_t)(or_uniform32(seed, (uint64_t)q + 1u, (int64_t)0xFFFFFFFFu, 0xFFFFFFFEu) < p);
}

/* Neumaier-compensated running sum: the sums of measures.jl:95-104 over millions of cells,
 * accurate to a few ulps whatever their order (the reference's own sum is pairwise, so no
 * order reproduces it bit for bit; an accurate sum is the fixed point both approximate). */
typedef struct { double s, c; } or_ksum;
static void or_ksum_add(or_ksum* k, double x) {
    double t = k->s + x;
    if (fabs(k->s) >= fabs(x)) k->c += (k->s - t) + x;
    else k->c += (x - t) + k->s;
    k->s = t;
}

double or_morans_i(const or_problem* P, const int8_t* u) {
    static const int vn[4][2] = {{0, -1}, {-1, 0}, {1, 0}, {0, 1}};
    int64_t n1 = P->n1, n2 = P->n2, n = n1 * n2;
    int64_t s = 0;
    for (int64_t k = 0; k < n; ++k) s += u[k];
    double m = (double)s / (double)n;
    or_ksum num = {0.0, 0.0};
    int64_t W = 0;
    for (int64_t j = 1; j <= n2; ++j)
        for (int64_t i = 1; i <= n1; ++i) {
            double xi = (double)u[(i - 1) + (j - 1) * n1] - m;
            for (int k = 0; k < 4; ++k) {
                int o1, o2;
                int64_t a = or_map_axis(P->boundary[0], i + vn[k][0], n1, &o1);
                int64_t b = or_map_axis(P->boundary[1], j + vn[k][1], n2, &o2);
                if (o1 || o2) continue; /* beyond a Constant edge: not a neighbour */
                or_ksum_add(&num, xi * ((double)u[(a - 1) + (b - 1) * n1] - m));
                W += 1;
            }
        }
    or_ksum den = {0.0, 0.0};
    for (int64_t k = 0; k < n; ++k) {
        double d = (double)u[k] - m;
        or_ksum_add(&den, d * d);
    }
    double dsum = den.s + den.c;
    if (dsum == 0.0) return NAN;
    return (double)n / (double)W * (num.s + num.c) / dsum;
}

/* ------------------------------------------------------------------ Lenia */

/* kernels.jl:96-104 */
static double or_lenia_value(double d, int32_t R, const double* peaks, int32_t B) {
    double r = d / (double)R;
    if (r <= 0.0 || r >= 1.0) return 0.0;
    double x = (double)B * r;
    int64_t i = (int64_t)floor(x);
    if (i > B - 1) i = B - 1;
    double f = x - (double)i;
    return (0.0 < f && f < 1.0) ? peaks[i] * exp(4.0 - 1.0 / (f * (1.0 - f))) : 0.0;
}

/* kernels.jl:174-189 then environment.jl:60-63 (negate the offsets). */
int or_lenia_weights(int32_t R, const double* peaks, int32_t npeaks, int32_t* off, double* w) {
    int m = 0;
    for (int dj = -R; dj <= R; ++dj)
        for (int di = -R; di <= R; ++di) {
            double d = sqrt((double)(di * di + dj * dj));
            if (!(d <= (double)R + 1e-9)) continue;
            double v = or_lenia_value(d, R, peaks, npeaks);
            if (v > 0.0) {
                off[2 * m] = -di;
                off[2 * m + 1] = -dj;
                w[m] = v;
                ++m;
            }
        }
    double s = 0.0;
    for (int k = 0; k < m; ++k) s += w[k];
    for (int k = 0; k < m; ++k) w[k] = w[k] / s;
    return m;
}

typedef struct {
    int64_t n1, n2;
    const int32_t* bnd;
    const void* cur;
    void* next;
    const int32_t* off;
    const double* w64;
    const float* w32;
    int m;
    double mu, sigma, dt;
    int f32;
    int64_t j0, j1;
} or_lenia_job;

static int64_t or_map_lenia(int32_t b, int64_t j, int64_t n, int* out) { return or_map_axis(b, j, n, out); }

static void* or_lenia_worker(void* arg) {
    or_lenia_job* L = (or_lenia_job*)arg;
    for (int64_t j = L->j0; j <= L->j1; ++j)
        for (int64_t i = 1; i <= L->n1; ++i) {
            int64_t lin = (i - 1) + (j - 1) * L->n1;
            if (!L->f32) {
                const double* u = (const double*)L->cur;
                double s = 0.0;
                for (int k = 0; k < L->m; ++k) {
                    int o1, o2;
                    int64_t a = or_map_lenia(L->bnd[0], i + L->off[2 * k], L->n1, &o1);
                    int64_t b = or_map_lenia(L->bnd[1], j + L->off[2 * k + 1], L->n2, &o2);
                    double x = (o1 || o2) ? 0.0 : u[(a - 1) + (b - 1) * L->n1];
                    s += L->w64[k] * x;
                }
                double c = u[lin];
                double d = s - L->mu;
                double g = 2.0 * exp(-(d * d) / (2.0 * (L->sigma * L->sigma))) - 1.0;
                double v = c + L->dt * g;
                v = v < 0.0 ? 0.0 : (v > 1.0 ? 1.0 : v);
                ((double*)L->next)[lin] = v;
            } else {
                const float* u = (const float*)L->cur;
                float s = 0.0f;
                for (int k = 0; k < L->m; ++k) {
                    int o1, o2;
                    int64_t a = or_map_lenia(L->bnd[0], i + L->off[2 * k], L->n1, &o1);
                    int64_t b = or_map_lenia(L->bnd[1], j + L->off[2 * k + 1], L->n2, &o2);
                    float x = (o1 || o2) ? 0.0f : u[(a - 1) + (b - 1) * L->n1];
                    s += L->w32[k] * x;
                }
                float mu = (float)L->mu, sg = (float)L->sigma, dt = (float)L->dt;
                float c = u[lin];
                float d = s - mu;
                float g = 2.0f * expf(-(d * d) / (2.0f * (sg * sg))) - 1.0f;
                float v = c + dt * g;
                v = v < 0.0f ? 0.0f : (v > 1.0f ? 1.0f : v);
                ((float*)L->next)[lin] = v;
            }
        }
    return NULL;
}

static int or_lenia_step(int64_t n1, int64_t n2, const int32_t* bnd, void* u, int f32, int32_t R,
                         const double* peaks, int32_t npeaks, double mu, double sigma, double dt,
                         int32_t nthreads) {
    int cap = (2 * R + 1) * (2 * R + 1);
    int32_t* off = (int32_t*)malloc(sizeof(int32_t) * 2 * (size_t)cap);
    double* w = (double*)malloc(sizeof(double) * (size_t)cap);
    float* w32 = (float*)malloc(sizeof(float) * (size_t)cap);
    size_t es = f32 ? sizeof(float) : sizeof(double);
    void* next = malloc(es * (size_t)(n1 * n2));
    if (!off || !w || !w32 || !next) { free(off); free(w); free(w32); free(next); return -2; }
    int m = or_lenia_weights(R, peaks, npeaks, off, w);
    for (int k = 0; k < m; ++k) w32[k] = (float)w[k];
    int nt = nthreads > 1 ? nthreads : 1;
    if (nt > n2) nt = (int)n2;
    pthread_t th[256];
    or_lenia_job jobs[256];
    if (nt > 256) nt = 256;
    for (int k = 0; k < nt; ++k) {
        or_lenia_job* L = &jobs[k];
        L->n1 = n1; L->n2 = n2; L->bnd = bnd; L->cur = u; L->next = next; L->off = off;
        L->w64 = w; L->w32 = w32; L->m = m; L->mu = mu; L->sigma = sigma; L->dt = dt; L->f32 = f32;
        L->j0 = (k * n2) / nt + 1;
        L->j1 = ((k + 1) * n2) / nt;
    }
    if (nt == 1) or_lenia_worker(&jobs[0]);
    else {
        for (int k = 0; k < nt; ++k) pthread_create(&th[k], NULL, or_lenia_worker, &jobs[k]);
        for (int k = 0; k < nt; ++k) pthread_join(th[k], NULL);
    }
    memcpy(u, next, es * (size_t)(n1 * n2));
    free(off); free(w); free(w32); free(next);
    return 0;
}

int or_lenia_step_f64(int64_t n1, int64_t n2, const int32_t* bnd, double* u, int32_t R,
                      const double* peaks, int32_t npeaks, double mu, double sigma, double dt,
                      int32_t nthreads) {
    return or_lenia_step(n1, n2, bnd, u, 0, R, peaks, npeaks, mu, sigma, dt, nthreads);
}

int or_lenia_step_f32(int64_t n1, int64_t n2, const int32_t* bnd, float* u, int32_t R,
                      const double* peaks, int32_t npeaks, double mu, double sigma, double dt,
                      int32_t nthreads) {
    return or_lenia_step(n1, n2, bnd, u, 1, R, peaks, npeaks, mu, sigma, dt, nthreads);
}

/* ------------------------------------------------------- dispersal kernels */

/* kernels.jl:30,47,64,78,96-104,126-132: unnormalised weight at distance d, offset (o1, o2). */
static double or_kernel_value(int32_t kind, double a, const double* peaks, int32_t npeaks, int32_t radius,
                              double d) {
    switch (kind) {
        case 1: return exp(-(d * d) / (2.0 * (a * a)));       /* Gaussian(sigma = a) */
        case 2: return exp(-d / a);                           /* Exponential(scale = a) */
        case 3: return pow(1.0 + d, -a);                      /* PowerLaw(alpha = a) */
        case 4: return 1.0;                                   /* Uniform */
        case 5: return or_lenia_value(d, radius, peaks, npeaks);
        default: return 0.0;
    }
}

int or_kernel_weights(int32_t kind, int32_t aniso_base, double a, double b, double c, int32_t radius,
                      const double* peaks, int32_t npeaks, const double* emp, int32_t emp_n1, int32_t emp_n2,
                      int32_t include_centre, int32_t* off, double* w) {
    int m = 0;
    if (kind == 7) {  /* kernels.jl:190-203: the matrix entries, centred, column-major */
        int c1 = (emp_n1 + 1) / 2, c2 = (emp_n2 + 1) / 2;
        for (int j = 1; j <= emp_n2; ++j)
            for (int i = 1; i <= emp_n1; ++i) {
                int o1 = i - c1, o2 = j - c2;
                if (o1 == 0 && o2 == 0 && !include_centre) continue;
                double v = emp[(i - 1) + (j - 1) * emp_n1];
                if (v > 0.0) { off[2 * m] = -o1; off[2 * m + 1] = -o2; w[m] = v; ++m; }
            }
    } else {
        for (int o2 = -radius; o2 <= radius; ++o2)
            for (int o1 = -radius; o1 <= radius; ++o1) {
                if (o1 == 0 && o2 == 0 && !include_centre) continue;
                double d = sqrt((double)(o1 * o1) + (double)(o2 * o2));   /* kernels.jl:154 */
                if (!(d <= (double)radius + 1e-9)) continue;
                double v;
                if (kind == 6) {   /* kernels.jl:126-132 */
                    v = or_kernel_value(aniso_base, a, peaks, npeaks, radius, d);
                    if (d != 0.0) {
                        /* Julia negates the Int offset: -0 is +0.0, so atan(0, x < 0) = +pi */
                        double th = atan2((double)(-o1), (double)o2);
                        v = v * exp(c * cos(th - b));
                    }
                } else {
                    v = or_kernel_value(kind, a, peaks, npeaks, radius, d);
                }
                if (v > 0.0) { off[2 * m] = -o1; off[2 * m + 1] = -o2; w[m] = v; ++m; }
            }
    }
    if (m == 0) return -1;
    double s = 0.0;
    for (int k = 0; k < m; ++k) s += w[k];
    for (int k = 0; k < m; ++k) w[k] = w[k] / s;
    return m;
}
