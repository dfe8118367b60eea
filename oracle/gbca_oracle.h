/*
 * gbca_oracle.h — CPU oracle for the synchronous halo-padded stencil sweep of
 * CellularAutomataCore.jl (ReferenceBackend / ArrayBackend semantics).
 *
 * TEST INFRASTRUCTURE ONLY. Nothing in the product library links, loads or
 * calls this code: only tests/, __graft_entry__.smoke() and bench.py's CPU
 * baseline / reference arm use it, as the checker. The reference package is
 * Julia, which is not installed here, so this is a restatement of its
 * algorithm in C; each function cites the reference file:line it follows.
 * It is pinned against the reference's own known-answer tests (Philox
 * vectors, rule definitions, classic patterns, scheme properties); see
 * tests/test_oracle.py.
 */
#ifndef GBCA_ORACLE_H
#define GBCA_ORACLE_H
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

enum { OR_RULE_LIFE = 1, OR_RULE_GENERATIONS = 2, OR_RULE_FOREST_FIRE = 3, OR_RULE_SI_FIELD = 5 };
enum { OR_MOORE = 1, OR_VON_NEUMANN = 2 };
enum { OR_PERIODIC = 0, OR_REFLECTING = 1, OR_CONSTANT = 2 };
enum { OR_SYNCHRONOUS = 0, OR_STOCHASTIC = 1, OR_CHECKERBOARD = 2 };

typedef struct or_problem {
    int32_t rule;          /* OR_RULE_* */
    int32_t nbhd;          /* OR_MOORE / OR_VON_NEUMANN */
    int32_t radius;
    int32_t states;        /* Generations C */
    uint64_t birth;        /* bit n: born with n live neighbours (rules.jl:267-275) */
    uint64_t survive;
    int64_t n1, n2;        /* dims; axis 1 contiguous (column-major) */
    int32_t boundary[2];   /* per axis */
    int32_t constant[2];   /* Constant value per axis (already an Int8 value) */
    uint64_t seed;
    int32_t scheme;        /* OR_SYNCHRONOUS / OR_STOCHASTIC / OR_CHECKERBOARD */
    int32_t scheme_p_f32;  /* Stochastic(p) with a Float32 p */
    double scheme_p;
    int32_t params_f32;    /* forest fire: p and f are Float32 */
    int32_t _pad;
} or_problem;

/* random.jl:24-37 */
void or_philox4x32(const uint32_t ctr[4], const uint32_t key[2], uint32_t out[4]);
/* random.jl:116-120 and :109-114 */
double or_uniform(uint64_t seed, uint64_t cellid, int64_t t, uint32_t k);
float or_uniform32(uint64_t seed, uint64_t cellid, int64_t t, uint32_t k);

/* neighbourhoods.jl:124-153: column-major offsets, centre excluded. Returns the
 * count; writes (di, dj) pairs into off (room for 2*(2r+1)^2 ints). */
int or_offsets(int32_t nbhd, int32_t radius, int32_t* off);

/* One full step t -> t+1 with ReferenceBackend semantics (backends.jl:264-278,
 * 314-322): boundary arithmetic on every neighbour read, serial. `params` is the
 * integrator's p (forest fire: {p, f}). cur is overwritten with the new state. */
int or_step_reference(const or_problem* P, int8_t* cur, int64_t t, const double* params);

/* nsteps steps from time t0 with ArrayBackend semantics (backends.jl:408-506):
 * halo-padded state, serial halo refresh, threaded slabs along the last axis.
 * nthreads <= 1 runs serially. state is updated in place. */
int or_run_array(const or_problem* P, int8_t* state, int64_t t0, int64_t nsteps,
                 const double* params, int32_t nthreads);

/* The environment of a sweep beyond the rule (environment.jl:82-148): a mask of cells
 * that update (environment.jl:123-130, backends.jl:448-450), one kernel field
 * (environment.jl:1-69,151-169) and one covariate layer (environment.jl:71-113).
 * The SI rule (OR_RULE_SI_FIELD) is the conformance battery's kernel-field epidemic
 * (test/backend_conformance.jl:52-57,72-75) as a typed rule: a cell in state 1 stays 1;
 * any other cell becomes 1 with probability 1 - exp(-beta * cov * field), draw k = 1,
 * where beta = params[0] (Float32 when P->params_f32), cov is the covariate at the cell
 * (slice mod1(t + 1, nt)) or absent, and field = sum_k w_k * (u[I + o_k] == 1) in tap
 * order, in Float32 when field_f32 (weights cast after FP64 normalisation). Products
 * follow Julia's promotion: Float32 with Float32 stays Float32, anything else is Float64. */
typedef struct or_env {
    const uint8_t* mask;     /* n1*n2, nonzero = the cell updates; NULL: no mask */
    int32_t ntaps;           /* kernel field taps; 0: no field */
    int32_t field_f32;
    const int32_t* taps;     /* offsets to read (already negated), (di, dj) pairs */
    const double* weights;   /* FP64 normalised weights */
    const void* cov;         /* n1*n2*cov_nt covariate values, or NULL */
    int64_t cov_nt;          /* slices along time (1: a fixed layer) */
    int32_t cov_f32;         /* covariate elements are Float32 */
    int32_t source;          /* field source: 0 = (x == 1), 1 = x itself */
} or_env;

/* kernels.jl:174-189 for the dispersal kernels of kernels.jl:1-152 on a square lattice,
 * then environment.jl:60-63 (negate the offsets). kind: 1 Gaussian(a = sigma),
 * 2 Exponential(a = scale), 3 PowerLaw(a = alpha), 4 Uniform, 5 Lenia(peaks),
 * 6 Anisotropic(base kind in aniso_base with a, direction b, strength c),
 * 7 Empirical (matrix `emp` of emp_n1 x emp_n2, column-major). Returns the tap count
 * written to off / w (room for (2*radius+1)^2), or -1 when no weight is positive. */
int or_kernel_weights(int32_t kind, int32_t aniso_base, double a, double b, double c, int32_t radius,
                      const double* peaks, int32_t npeaks, const double* emp, int32_t emp_n1, int32_t emp_n2,
                      int32_t include_centre, int32_t* off, double* w);

/* environment.jl:151-160: the field of every cell of u, into f64 (and its
 * Float32 counterpart into f32 when E->field_f32); both arrays hold n1*n2 values. */
int or_kernel_field(const or_problem* P, const or_env* E, const int8_t* u, double* f64, float* f32);

/* or_step_reference / or_run_array with an environment (NULL = none). */
int or_step_reference_env(const or_problem* P, const or_env* E, int8_t* cur, int64_t t, const double* params);
int or_run_array_env(const or_problem* P, const or_env* E, int8_t* state, int64_t t0, int64_t nsteps,
                     const double* params, int32_t nthreads);

/* measures.jl:14-20: counts[v] for v in 0..nvals-1 (values outside are ignored,
 * *other receives their number). */
void or_state_counts(const int8_t* u, int64_t n, int64_t* counts, int32_t nvals, int64_t* other);

/* measures.jl:91-107 with neighbourhood VonNeumann(1) on the problem's lattice
 * (boundaries from P). Returns NaN for a constant field (the reference raises). */
double or_morans_i(const or_problem* P, const int8_t* u);

/* The Bernoulli(density) soup of 0/1 the backend generates on the device for a state it is
 * not given (no counterpart in the reference): cell q (1-based column-major id) is 1 when the
 * Float32 uniform of its draw (seed; q, 0, 0xFFFFFFFF, 0xFFFFFFFE) (random.jl:102-114) lies
 * below Float32(density), as bernoulli(Float32) compares (random.jl:130). */
void or_soup(uint64_t seed, int64_t n1, int64_t n2, double density, int8_t* out);

/* Lenia (lenia.jl:42-47, environment.jl:151-169, kernels.jl:87-104,174-189).
 * or_lenia_weights: offsets to read (negated kernel offsets, column-major order)
 * and FP64-normalised weights; returns the tap count (room for (2R+1)^2). */
int or_lenia_weights(int32_t R, const double* peaks, int32_t npeaks, int32_t* off, double* w);
/* One Lenia step on a Float64 state with FP64 field (ReferenceBackend semantics,
 * boundary reads per access), threaded over cells. */
int or_lenia_step_f64(int64_t n1, int64_t n2, const int32_t* bnd, double* u, int32_t R,
                      const double* peaks, int32_t npeaks, double mu, double sigma, double dt,
                      int32_t nthreads);
/* The same with precision=Float32 (weights cast to Float32 after FP64
 * normalisation, field and growth in Float32, no fused multiply-add). */
int or_lenia_step_f32(int64_t n1, int64_t n2, const int32_t* bnd, float* u, int32_t R,
                      const double* peaks, int32_t npeaks, double mu, double sigma, double dt,
                      int32_t nthreads);

#ifdef __cplusplus
}
#endif
#endif
