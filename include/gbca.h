/*
 * gbca.h — C ABI of libgbca.so, the GB300 (sm_103a) backend for the synchronous
 * halo-padded stencil sweep of CellularAutomataCore.jl.
 *
 * Each entry point replaces one method of the reference's backend contract
 * (src/backends.jl:4-14, declared `public` in src/CellularAutomataCore.jl:257), as the
 * KernelAbstractions GPUBackend implements it (ext/CellularAutomataCoreKernelAbstractionsExt.jl).
 * Plain C types only: pointers, sizes, fixed-width integers and doubles. No exception
 * crosses the ABI: every call returns a status (GBCA_OK = 0) and gbca_last_error() gives
 * the message of the calling thread's last failure.
 *
 * States are single-layer, column-major (axis 1 contiguous), exactly the layout of the
 * reference's `u0` arrays: Int8 for Life / Generations / forest fire, Float32 or Float64
 * for Lenia.
 * Indices are 1-based, as in Julia. A handle owns its device buffers and one CUDA stream;
 * a handle is not thread-safe, distinct handles are.
 */
#ifndef GBCA_H
#define GBCA_H

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

/* ---- status codes; the host glue maps them to the reference's exception types */
#define GBCA_OK 0
#define GBCA_ERR_ARGUMENT 1            /* ArgumentError */
#define GBCA_ERR_INCOMPATIBLE_SPACE 2  /* IncompatibleSpaceError (src/errors.jl) */
#define GBCA_ERR_UNSUPPORTED 3         /* UnsupportedCombinationError (src/errors.jl:124-132) */
#define GBCA_ERR_STATE 4               /* StateShapeError / InvalidStateError */
#define GBCA_ERR_CUDA 5                /* a CUDA runtime or cuFFT failure */
#define GBCA_ERR_OUT_OF_MEMORY 6       /* device memory or an HBM budget is exhausted */
#define GBCA_ERR_TIMEOUT 7             /* a bounded device-side wait gave up */
#define GBCA_ERR_BUSY 8                /* a queue is full; retry later */

/* ---- problem description (what check_problem / allocate_state receive as `prob`) */
enum { GBCA_RULE_LIFE = 1, GBCA_RULE_GENERATIONS = 2, GBCA_RULE_FOREST_FIRE = 3, GBCA_RULE_LENIA = 4,
       GBCA_RULE_SI_FIELD = 5 };
enum { GBCA_SOURCE_INDICATOR = 0, GBCA_SOURCE_IDENTITY = 1 };
enum { GBCA_MOORE = 1, GBCA_VON_NEUMANN = 2 };
enum { GBCA_PERIODIC = 0, GBCA_REFLECTING = 1, GBCA_CONSTANT = 2 };
enum { GBCA_SYNCHRONOUS = 0, GBCA_STOCHASTIC = 1, GBCA_CHECKERBOARD = 2 };
enum { GBCA_DIRECT = 0, GBCA_FFT = 1 };
enum { GBCA_INT8 = 1, GBCA_FLOAT32 = 2 };

#define GBCA_MAX_PEAKS 8

typedef struct gbca_desc {
    int32_t rule;            /* GBCA_RULE_*                                         */
    int32_t nbhd;            /* GBCA_MOORE / GBCA_VON_NEUMANN (src/neighbourhoods.jl:21,35) */
    int32_t radius;          /* neighbourhood radius r >= 1                          */
    int32_t states;          /* Generations: C (src/rules.jl:424-429)               */
    uint64_t birth;          /* Life / Generations masks: bit n <=> count n (rules.jl:267-275) */
    uint64_t survive;
    int64_t n1, n2;          /* lattice dims (src/spaces.jl:94-110)                  */
    int32_t boundary[2];     /* GBCA_PERIODIC / GBCA_REFLECTING / GBCA_CONSTANT per axis */
    double constant[2];      /* the Constant(value) of each axis                     */
    uint64_t seed;           /* prob.seed (src/problem.jl:90)                        */
    int32_t scheme;          /* GBCA_SYNCHRONOUS / GBCA_STOCHASTIC / GBCA_CHECKERBOARD */
    int32_t scheme_p_f32;    /* Stochastic(p) with a Float32 p (schemes.jl:86-88)     */
    double scheme_p;
    int32_t params_f32;      /* forest fire: p and f are Float32 (random.jl:130)     */
    int32_t lenia_method;    /* GBCA_DIRECT / GBCA_FFT (src/lenia.jl:24-32)          */
    int32_t lenia_R;
    int32_t lenia_npeaks;
    int32_t lenia_f64;       /* Lenia(; precision=Float64): a Float64 state (src/lenia.jl:24-31) */
    int32_t reserved;
    double lenia_peaks[GBCA_MAX_PEAKS];
    double lenia_mu, lenia_sigma, lenia_dt;
} gbca_desc;

typedef struct gbca_handle gbca_handle;

/* Message of the calling thread's last failed call ("" if none). */
const char* gbca_last_error(void);

/* Library version: major * 10000 + minor * 100 + patch. */
int32_t gbca_version(void);

/* Number of CUDA devices (0 without a GPU); never fails. */
int32_t gbca_device_count(void);

/* Replaces check_problem(b, prob, scheme) (src/backends.jl:97-105; the KA version
 * ext/CellularAutomataCoreKernelAbstractionsExt.jl:42-49). Validates a description
 * without touching the GPU. */
int gbca_check(const gbca_desc* desc);

/* Replaces allocate_state(b, prob, scheme) (src/backends.jl:107-119; KA ext :51-59):
 * checks the description, allocates the device state on the current device and zeroes
 * it. The caller then uploads prob.u0 with gbca_set_state. */
int gbca_create(const gbca_desc* desc, gbca_handle** out);

/* Frees the device buffers and the stream. */
int gbca_destroy(gbca_handle* h);

/* Replaces set_state!(b, st, u) (src/backends.jl:141-148; KA ext :132-140): copies a
 * whole host state (n1*n2 elements, column-major) to the device. */
int gbca_set_state(gbca_handle* h, const void* host, size_t nbytes);

/* set_state! from a state already in device memory (a CuArray, say): `dptr` holds n2
 * columns of n1 elements, `src_pitch` bytes apart (n1 * element size when packed). The
 * copy is queued on the handle's stream. */
int gbca_set_state_device(gbca_handle* h, const void* dptr, int64_t src_pitch);

/* set_state! with a Bernoulli(density) soup of 0/1 generated on the device from `seed` (cell
 * id's draw (seed; id, 0, 0xFFFFFFFF, 0xFFFFFFFE) as a Float32 uniform), the same generator
 * gbca_server_submit uses for requests without a state. Queued on the handle's stream.
 * No counterpart in the reference (its initial states come from the host). */
int gbca_set_state_soup(gbca_handle* h, double density, uint64_t seed);

/* Replaces current_state(b, st) (src/backends.jl:132-139; KA ext :126-130): waits for
 * pending work and copies the whole state to host memory. */
int gbca_get_state(gbca_handle* h, void* host, size_t nbytes);

/* gbca_set_state and gbca_get_state without the wait: the copy is queued on the handle's stream
 * (after the work queued before it) and the call returns at once, so a caller can overlap one
 * lattice's copies with another's sweeps, or one step's result with the next step's input.
 * The host buffer should be page-locked (pinned; otherwise the driver stages it and the copy
 * is not asynchronous) and must be left untouched until the copy has run: until gbca_sync(h)
 * or any call that waits on the handle's stream. The reference's set_state! and
 * current_state (src/backends.jl:132-148) are synchronous; these are their queued forms. */
int gbca_set_state_async(gbca_handle* h, const void* host, size_t nbytes);
int gbca_get_state_async(gbca_handle* h, void* host, size_t nbytes);

/* Replaces advance!(b, st, prob, scheme, p, t) (src/backends.jl:121-130; KA ext :92-110),
 * `nsteps` times: the state goes from time t to t + nsteps. `params` is the integrator's
 * p: forest fire {p, f}; the kernel-field SI rule {beta}; unused otherwise (may be NULL
 * with nparams = 0). The SI rule (GBCA_RULE_SI_FIELD) is the conformance battery's
 * kernel-field epidemic (test/backend_conformance.jl:52-57,72-75) as a typed rule: a cell
 * in state 1 stays 1, any other becomes 1 when bernoulli(ctx, 1 - exp(-beta * cov * field))
 * (draw k = 1), with cov the covariate (or none) and field the kernel field; params_f32
 * makes beta Float32, and products promote as in Julia. Work is queued
 * on the handle's stream; the call returns before it finishes. */
int gbca_advance(gbca_handle* h, int64_t t, int64_t nsteps, const double* params, int32_t nparams);

/* Replaces read_cell(b, st, I) (src/backends.jl:380; KA ext :142): one element at the
 * 1-based index (i, j), written to `out` (1 byte for Int8, 4 for Float32, 8 for Float64). */
int gbca_read_cell(gbca_handle* h, int64_t i, int64_t j, void* out);

/* Replaces write_cell!(b, st, I, v) (src/backends.jl:381-383; KA ext :143-148). */
int gbca_write_cell(gbca_handle* h, int64_t i, int64_t j, const void* value);

/* ---- the environment of a sweep (src/environment.jl:82-148), attached after gbca_create.
 *
 * Replaces CAProblem's `mask` (problem.jl:20-27, environment.jl:123-130): cells whose byte is
 * 0 never update, though their neighbours still read them (backends.jl:448-450). `host` holds
 * n1*n2 bytes, column-major, nonzero = the cell updates; NULL removes the mask. Int8 rules
 * only (GBCA_ERR_UNSUPPORTED for Lenia). A masked forest fire runs its fast kernel one step per
 * launch; masked Life and Generations of radius <= 2 (Moore) or von Neumann(1) run the
 * bit-sliced kernel with the mask as a bit plane; other masked problems the general kernel. */
int gbca_set_mask(gbca_handle* h, const uint8_t* host, size_t nbytes);

/* Replaces the resolved KernelField of a GBCA_RULE_SI_FIELD problem (environment.jl:53-69):
 * `taps` holds ntaps (di, dj) offsets to READ (kernel_weights' offsets negated, in its order),
 * `weights` their FP64-normalised weights (kernels.jl:174-189); f32 = 1 for
 * precision = Float32 (weights cast after normalising, sum in Float32); source is
 * GBCA_SOURCE_INDICATOR (x == 1) or GBCA_SOURCE_IDENTITY (x); method GBCA_DIRECT (taps
 * within radius 64) or GBCA_FFT (periodic boundaries on both axes; the field agrees with
 * the direct sum to rounding, as ext/CellularAutomataCoreFFTWExt.jl does). */
int gbca_set_field(gbca_handle* h, int32_t ntaps, const int32_t* taps, const double* weights, int32_t f32,
                   int32_t source, int32_t method);

/* Replaces the covariate a GBCA_RULE_SI_FIELD rule reads (environment.jl:71-113): n1*n2*nt
 * values, column-major, time last (slice mod1(t + 1, nt) at time t; nt = 1 for a fixed
 * layer), Float64 (f32 = 0) or Float32 (f32 = 1); NULL removes it. */
int gbca_set_covariate(gbca_handle* h, const void* host, int64_t nt, int32_t f32);

/* ---- active-tile scheduling: the GPU form of SparseBackend(background; tilesize)
 * (src/sparse.jl:1-211). With enable = 1, each sweep runs only the tiles (tilesize x tilesize
 * cells; 0 = 64) that hold a cell other than `background` or lie within reach of one, for
 * quiescent rules: a background cell with background neighbours must stay background (Life
 * without B0 on background 0, Generations on 0, the forest fire with p = 0 on empty or f = 0 on
 * trees); GBCA_ERR_ARGUMENT otherwise (the forest fire is checked at each gbca_advance, whose
 * parameters decide it). Synchronous and Stochastic only, as SparseBackend (sparse.jl:40);
 * masks allowed. Results equal the dense sweep's. enable = 0 returns to dense sweeps. */
int gbca_set_sparse(gbca_handle* h, int32_t enable, int32_t background, int32_t tilesize);

/* ---- the device-side save path: saved states staged on the device and copied out
 * asynchronously through pinned buffers, so saveat does not stall the sweep.
 * No counterpart in the reference (its integrator copies each saved state synchronously,
 * src/problem.jl:336-370). */
#define GBCA_MAX_SNAPSHOTS 64

/* Queues a copy of the state as it will be after the work queued so far: a device-to-device
 * copy on the handle's stream, then a device-to-host copy into pinned memory on a second
 * stream. Returns at once with a ticket for gbca_snapshot_fetch. At most GBCA_MAX_SNAPSHOTS
 * may wait to be fetched (GBCA_ERR_BUSY beyond). */
int gbca_snapshot(gbca_handle* h, int64_t* ticket);

/* Waits for snapshot `ticket` and copies it (column-major, n1*n2 elements) to `host`. */
int gbca_snapshot_fetch(gbca_handle* h, int64_t ticket, void* host, size_t nbytes);

/* Waits for the handle's queued work. */
int gbca_sync(gbca_handle* h);

/* state_counts (src/measures.jl:14-20) and Moran's I with VonNeumann(1) on the problem's
 * lattice (src/measures.jl:91-107), computed on the device from the current Int8 state.
 * counts[v] for v in 0..nvals-1; *other gets the number of cells outside that range.
 * *morans is NaN for a constant field (where the reference raises ArgumentError). */
int gbca_summaries(gbca_handle* h, int64_t* counts, int32_t nvals, int64_t* other, double* morans);

/* Device pointer of the current state buffer (pitch in bytes between columns in *pitch),
 * valid until the next gbca_advance / gbca_destroy. For callers that keep inputs in HBM. */
int gbca_device_state(gbca_handle* h, void** dptr, int64_t* pitch);

/* The handle's lattice (n1 x n2) as columns col0 .. col0 + n2 - 1, taken modulo n2_global, of a
 * lattice of n1 x n2_global cells: the slab one rank holds when the single sweep is split along
 * its last axis, as ArrayBackend's threads split it (src/backends.jl:457-479). Cell ids (hence
 * every draw, random.jl:102-107) and Checkerboard parities (schemes.jl:89) become the larger
 * lattice's; neighbours are still read from the handle's own lattice through its boundaries, so
 * a caller that pads the slab with h = r x steps x gates columns on each side the larger lattice
 * continues and refreshes them every `steps` steps gets exact owned columns. col0 = 0 with
 * n2_global = n2 restores a lattice of its own. Int8 rules only (Life, Generations, forest fire),
 * dense sweeps only (no gbca_set_sparse); needs -n2_global < col0 < n2_global. */
int gbca_set_slab(gbca_handle* h, int64_t col0, int64_t n2_global);

/* The exact integer sums behind state_counts and Moran's I (src/measures.jl:14-20,91-107) over
 * the cells of columns j_lo .. j_hi - 1 of the current state, neighbours read through the
 * handle's boundaries: sums[0..255] count the values -128..127, then S = sum x, S2 = sum x^2,
 * P = sum over VonNeumann(1) neighbour pairs of x_i x_j, Q = sum over pairs of x_i + x_j, and
 * W = the number of pairs (261 values). Slabs' sums add up to the whole lattice's, from which
 * Moran's I = (n^2 P - n S Q + W S^2) / (W (n S2 - S^2)). */
int gbca_slab_sums(gbca_handle* h, int64_t j_lo, int64_t j_hi, int64_t* sums);

/* Run the handle's work on `stream` (a cudaStream_t; NULL restores the handle's own
 * stream) from the next call on, after waiting for what was queued before. Lets a caller
 * order the sweep with its own work and time it with events on the same stream.
 * No counterpart in the reference (its GPUBackend synchronizes after every step). */
int gbca_set_stream(gbca_handle* h, void* stream);

/* Number of kernels this library has launched in the process so far (all handles).
 * A diagnostic with no counterpart in the reference. */
int64_t gbca_kernel_launches(void);

/* Measured compute roof of the stochastic sweeps: Philox4x32-10 cell draws per second
 * (random.jl:102-107 with the bernoulli compare of random.jl:129) when the GPU does nothing
 * else, over about `draws` draws on the legacy default stream. The forest-fire rule makes one
 * draw per cell-update. A diagnostic with no counterpart in the reference. */
int gbca_philox_rate(int64_t draws, double* draws_per_s);

/* Self-test of the failure path of the device-side waits: one kernel waits, at most `polls`
 * polls (1..2^20), on a barrier that nothing completes, and records the timeout as a tile copy
 * that gave up would. Returns GBCA_ERR_TIMEOUT, read on the host; the context stays usable.
 * Nothing faults, traps or hangs. No counterpart in the reference. */
int gbca_selftest_wait(int32_t polls);

/* ---- sweep autotuning. No counterpart in the reference (its kernels have one geometry).
 * A sweep geometry is (steps per temporally blocked pass, tile rows, tile staging). gbca_tune
 * times every candidate geometry of the handle's fast kernel (forest fire: pass depth x
 * staging by vector loads or by TMA; bit-sliced Life/Generations: pass depth x tile height) on
 * the handle's current state, about 48 steps each, restores the state, and caches the fastest
 * for the problem's shape (rule, neighbourhood, size, boundaries, scheme, device): every later
 * sweep of that shape, on any handle or in the server, uses it. The chosen geometry is
 * returned ((0, 0, 0): the problem runs on the general kernel, nothing to tune; staging may be
 * NULL). Results never depend on the geometry. It allocates one copy of the state while it
 * runs; params as in gbca_advance. */
int gbca_tune(gbca_handle* h, const double* params, int32_t nparams, int32_t* steps_per_pass, int32_t* tile_rows,
              int32_t* staging);

/* The geometry the handle's next sweep uses (pinned, tuned or the kernel's default), (0, 0, 0)
 * for the general kernel, Lenia, the SI rule and active-tile sweeps. params as in gbca_advance
 * (the forest fire's decide whether its fast kernel applies). */
int gbca_geometry(gbca_handle* h, const double* params, int32_t* steps_per_pass, int32_t* tile_rows,
                  int32_t* staging);

/* Clears the tuning cache (all shapes). */
int gbca_forget_tuning(void);

/* Pins this handle's sweep geometry ((0, 0, 0) unpins it). The forest-fire kernel takes
 * tile_rows 0 (its launcher's model) or 8..240 rows whose tiles fit shared memory, and
 * staging 0 (vector loads), 1 (a TMA copy per tile where the tile fits) or
 * 2 (the same, prefetched by a persistent kernel; one step per pass only); the bit-sliced
 * kernel takes tile_rows 0 (its default) or any height whose tiles fit shared memory, and
 * staging 0; the general kernel takes none (GBCA_ERR_UNSUPPORTED). */
int gbca_set_geometry(gbca_handle* h, int32_t steps_per_pass, int32_t tile_rows, int32_t staging);

/* ---- batched ensembles: many problems advanced by one persistent, graph-captured launch.
 * Replaces solving an EnsembleProblem one trajectory at a time (src/problem.jl:571-589 with
 * SciMLBase's EnsembleSerial / EnsembleThreads; src/calibration.jl:66-91 for ABC): each
 * instance is its own gbca_desc (its size, rule, boundaries and seed — seed_trajectory gives
 * trajectory i the seed prob.seed + i), Int8 rules, Synchronous, radius <= 8. */
typedef struct gbca_ensemble gbca_ensemble;

/* Allocates every instance's two state buffers (zeroed) in one pool. */
int gbca_ensemble_create(const gbca_desc* descs, int32_t n, gbca_ensemble** out);
int gbca_ensemble_destroy(gbca_ensemble* e);

/* Initial state of instance i (n1*n2 bytes, column-major), or every cell of every instance. */
int gbca_ensemble_set_state(gbca_ensemble* e, int32_t i, const void* host, size_t nbytes);
int gbca_ensemble_fill(gbca_ensemble* e, int32_t value);

/* Advances instance i by nsteps[i] steps from time t0[i] (t0 may be NULL for 0), with its
 * parameters at params[i * nparams ...] (forest fire: p, f). One graph launch; queued. At the
 * end of the run every instance's state counts and Moran's I sums are computed on the device. */
int gbca_ensemble_run(gbca_ensemble* e, const int64_t* t0, const int64_t* nsteps, const double* params,
                      int32_t nparams);
int gbca_ensemble_sync(gbca_ensemble* e);

/* state_counts and Moran's I (src/measures.jl:14-20,91-107) of every instance's state at the
 * end of the last run: counts[i * nvals + v] for v < nvals <= 8, other[i], morans[i] (NaN for a
 * constant field). The same integers, hence the same bits, as gbca_summaries on one handle. */
int gbca_ensemble_summaries(gbca_ensemble* e, int64_t* counts, int32_t nvals, int64_t* other, double* morans);

/* current_state of instance i. */
int gbca_ensemble_get_state(gbca_ensemble* e, int32_t i, void* host, size_t nbytes);

/* The ensemble kernel's geometry: tiles of `tile` cells a side (64, 128 or 192; the shared
 * buffers, hence which lattices live whole in shared memory, follow the tile) and `depth`
 * steps per temporally blocked pass of the tiled path (1..8, 0 = the deepest the halo of 8
 * cells allows for the instance's radius). Results never depend on it. No counterpart in the
 * reference. */
int gbca_ensemble_set_geometry(gbca_ensemble* e, int32_t tile, int32_t depth);

/* Which instances leave the persistent kernel: forest-fire instances (VonNeumann(1)) of at
 * least min_cells cells (0 = none; else at least 2^14) run as batched multi-CTA passes — every
 * tile of every such instance in one launch, steps_per_pass (1..16) steps per launch — on a
 * second stream of the same graph, and their summaries by a batched reduction. Default 2^18
 * cells, 1 step per pass. Results never depend on it. No counterpart in the reference. */
int gbca_ensemble_set_large(gbca_ensemble* e, int64_t min_cells, int32_t steps_per_pass);

/* The geometry the next run uses (any pointer may be NULL); n_large = instances that run as
 * batched passes. */
int gbca_ensemble_geometry(gbca_ensemble* e, int32_t* tile, int32_t* depth, int64_t* large_cells,
                           int32_t* large_steps, int32_t* n_large);

/* The autotuner for the batched path: times every (tile, depth) candidate on the ensemble's
 * own instances for `probe_steps` steps each from their current states (restored after every
 * candidate and at the end; params as in gbca_ensemble_run), keeps the fastest, then times the
 * large-instance split (min_cells 2^14 .. 2^18, 2^20 or none x 1, 2 or 4 steps per pass)
 * where an instance could take it, and keeps the fastest of all; returns tile and depth
 * (gbca_ensemble_geometry gives the rest). It allocates one copy of the ensemble's state pool
 * while it runs; summaries are those of the last probe until the next gbca_ensemble_run. No
 * counterpart in the reference. */
int gbca_ensemble_tune(gbca_ensemble* e, int64_t probe_steps, const double* params, int32_t nparams, int32_t* tile,
                       int32_t* depth);

/* ---- serving: a device-resident request loop with continuous batching. Clients submit
 * simulation requests at any time; a scheduler thread admits them in arrival order while
 * their state buffers fit the HBM budget and returns each request's state counts and Moran's
 * I as soon as it finishes. Small requests advance together in persistent launches, up to
 * chunk_steps steps each per launch (fewer on larger lattices, so a launch stays short); large ones (above big_cells cells) run as multi-CTA sweeps on up to max_big stream
 * lanes, in chunks of big_chunk_us of estimated GPU time (at least chunk_steps steps),
 * the request with the shortest estimated remaining time (less its time in the system) first,
 * while the chunks in flight fill at most two GPUs' worth of tiles. A request's result does
 * not depend on what else runs. No counterpart in the reference (its unit of work is one
 * solve at a time). */
typedef struct gbca_server gbca_server;

typedef struct gbca_server_config {
    uint64_t hbm_budget;   /* bytes of device memory for request states (two buffers each) */
    int32_t chunk_steps;   /* steps per request per iteration */
    int32_t big_cells;     /* requests above this many cells run as their own multi-CTA sweeps */
    int32_t max_big;       /* large requests advanced concurrently (one stream each), 1..64 */
    int32_t big_chunk_us;  /* a large request's chunk, in microseconds of estimated GPU time (at least
                              chunk_steps steps); 0 = 4000 */
} gbca_server_config;

typedef struct gbca_result {
    uint64_t id;
    int32_t status;        /* GBCA_OK, or GBCA_ERR_OUT_OF_MEMORY for a request larger than the budget */
    int32_t reserved;
    int64_t counts[8];     /* cells holding 0..7 */
    int64_t other;         /* cells holding any other value */
    double morans;         /* Moran's I, VonNeumann(1) on the request's lattice; NaN if constant */
    double t_submit, t_admit, t_done;  /* seconds on the server's clock */
} gbca_result;

int gbca_server_start(const gbca_server_config* cfg, gbca_server** out);

/* Queue a request: an Int8 problem (Synchronous, radius <= 8), its initial state (u0: n1*n2
 * bytes, column-major; or NULL for a Bernoulli(init_density) soup of 0/1 drawn from
 * init_seed on the device, all zeros for density 0), nsteps steps from time t0, parameters
 * (forest fire: p, f). Returns at once with the request's id. */
int gbca_server_submit(gbca_server* s, const gbca_desc* d, const void* u0, size_t nbytes, double init_density,
                       uint64_t init_seed, int64_t t0, int64_t nsteps, const double* params, int32_t nparams,
                       uint64_t* id);

/* Up to `max` finished requests' results, oldest first; *n gets how many. Never blocks. */
int gbca_server_poll(gbca_server* s, gbca_result* out, int32_t max, int32_t* n);

/* Requests waiting for admission, requests admitted, and the server's clock (seconds). */
int gbca_server_status(gbca_server* s, int64_t* queued, int64_t* active, double* clock);

/* Occupancy so far: the seconds each large-request lane had a chunk in flight
 * (lane_busy_s[0 .. min(max_lanes, lanes) - 1]; *nlanes gets the number of lanes), the seconds
 * the small requests' stream had a launch in flight, the server's clock, and the number of
 * large-request chunks run. Any output but lane_busy_s may be NULL. No counterpart in the
 * reference. */
int gbca_server_stats(gbca_server* s, double* lane_busy_s, int32_t max_lanes, int32_t* nlanes, double* small_busy_s,
                      double* wall_s, int64_t* chunks);

/* Stop accepting requests, finish every queued and admitted one, free everything.
 * Results not yet polled are lost. */
int gbca_server_stop(gbca_server* s);

/* Size of the device scratch array behind gbca_advance_noalloc: the largest state, in bytes
 * (pitch * n2), that it accepts. Every GPU that loads the library holds this array until
 * the process exits. */
#define GBCA_NOALLOC_SCRATCH_BYTES (16 * 1024 * 1024)

/* gbca_advance for callers that cannot allocate device memory when they need a sweep: code
 * running while a memory pool owns the device (a CuArray pool, a caching allocator sized to
 * the card), a real-time loop that must not take the allocator's locks, or a plug-in whose
 * host forbids allocation after start-up. No counterpart in the reference.
 *
 * Advances the Int8 state at `state` (n2 columns of desc->n1 bytes, `pitch` bytes apart,
 * 16-byte aligned, pitch a multiple of 16 for the fast kernels) by `nsteps` steps from time
 * t, in place, on `stream` (a cudaStream_t; NULL is the legacy default stream). It allocates
 * nothing and creates no stream: the buffer the sweep alternates with is a file-scope device
 * array of GBCA_NOALLOC_SCRATCH_BYTES; larger states are refused with GBCA_ERR_ARGUMENT, and
 * Lenia (whose FFT plans allocate) with GBCA_ERR_UNSUPPORTED. Results are those of
 * gbca_advance, bit for bit. The work is queued; the call returns before it finishes.
 *
 * The sweep is gbca_advance's own (same kernels, geometry and staging). The state is not
 * scanned first, so Generations, and Life under a gate or a mask, take the general kernel
 * (slower than the bit-sliced one it would reach on a handle, same results).
 *
 * The first call on a device looks up the scratch array's address in the calling thread's
 * current CUDA context (make it before any stream capture on that device); the address is
 * kept per context, and a context created anew (after cudaDeviceReset) is looked up again.
 * All calls share the array and it keeps the last call's contents: calls that overlap on
 * the GPU race on it, so serialise them. */
int gbca_advance_noalloc(const gbca_desc* desc, void* state, int64_t pitch, int64_t t, int64_t nsteps,
                         const double* params, int32_t nparams, void* stream);

/* Host helper: the integer threshold T with  uniform < p  <=>  x < T, where x is the
 * 53-bit (f32 = 0: random.jl:116-120) or 24-bit (f32 = 1: random.jl:109-114) integer
 * behind the draw. NaN and p <= 0 give 0; p >= 1 gives 2^53 (2^24). */
uint64_t gbca_threshold(double p, int32_t f32);

#ifdef __cplusplus
}
#endif
#endif
