// gbca_internal.cuh — device helpers shared by the sweep kernels of libgbca.so:
// the counter-based Philox4x32-10 draws keyed as src/random.jl:102-107, the
// boundary mapping of src/spaces.jl:46-51, and the launch parameters of a sweep.
#pragma once

#include <vector>

#include <cstdint>
#include <cuda_runtime.h>

#include "gbca.h"

namespace gbca {

// ----------------------------------------------------------------- Philox4x32-10

constexpr uint32_t kPhM0 = 0xD2511F53u;
constexpr uint32_t kPhM1 = 0xCD9E8D57u;
constexpr uint32_t kPhW0 = 0x9E3779B9u;
constexpr uint32_t kPhW1 = 0xBB67AE85u;

// The 64-bit product m * c as its high and low words, by two 32-bit multiplies (mul.hi.u32,
// mul.lo.u32). The same bits as one 32x32->64 multiply; on GB300 a Philox4x32-10 draw built
// from this form runs at 492 Gdraws/s against 428 for the 64-bit form (all SMs, one chain per
// thread, 2048 threads per SM).
__device__ __forceinline__ void mul_hilo(uint32_t m, uint32_t c, uint32_t& hi, uint32_t& lo) {
    asm("mul.hi.u32 %0, %1, %2;" : "=r"(hi) : "r"(m), "r"(c));
    asm("mul.lo.u32 %0, %1, %2;" : "=r"(lo) : "r"(m), "r"(c));
}

// Words 1 and 2 of philox4x32(ctr, key) (src/random.jl:24-37): ten rounds, the key
// bumped after rounds 1..9. Only words 1 and 2 feed the draws (random.jl:109-120),
// so round 10 needs one of its two products.
__device__ __forceinline__ uint2 philox_w01(uint32_t c0, uint32_t c1, uint32_t c2, uint32_t c3,
                                            uint32_t k0, uint32_t k1) {
#pragma unroll
    for (int r = 0; r < 9; ++r) {
        uint32_t h0, l0, h1, l1;
        mul_hilo(kPhM0, c0, h0, l0);
        mul_hilo(kPhM1, c2, h1, l1);
        const uint32_t n0 = h1 ^ c1 ^ k0, n2 = h0 ^ c3 ^ k1;
        c0 = n0; c1 = l1; c2 = n2; c3 = l0;
        k0 += kPhW0; k1 += kPhW1;
    }
    uint32_t h1, l1;
    mul_hilo(kPhM1, c2, h1, l1);
    return make_uint2(h1 ^ c1 ^ k0, l1);
}

// The draw of cell `id` (1-based column-major linear index, backends.jl:446) at time t
// with draw index k: counter (id lo, id hi, t mod 2^32, k), key (seed lo, seed hi).
__device__ __forceinline__ uint2 cell_draw(uint64_t seed, uint64_t id, int64_t t, uint32_t k) {
    return philox_w01((uint32_t)id, (uint32_t)(id >> 32), (uint32_t)(uint64_t)t, k,
                      (uint32_t)seed, (uint32_t)(seed >> 32));
}

// uniform(...) < p, evaluated exactly as an integer compare against a host-computed
// threshold: for a Float64 p the 53-bit integer x of random.jl:118-119, for a Float32 p
// the 24-bit integer of random.jl:111.
__device__ __forceinline__ bool draw_below(uint2 w, uint64_t thr, bool f32) {
    if (f32) return (uint64_t)(w.x >> 8) < thr;
    return ((((uint64_t)w.x << 32) | (uint64_t)w.y) >> 11) < thr;
}

// The ten round keys of a seed: (seed lo + r W0, seed hi + r W1), r = 0..9 (random.jl:31-33).
// Passed in the kernel parameters, so each key XOR is one three-input LOP3 with a
// parameter-bank operand instead of a per-thread running sum.
struct PhiloxKeys {
    uint32_t k0[10], k1[10];
};

__host__ __device__ inline PhiloxKeys philox_keys(uint64_t seed) {
    PhiloxKeys K;
    uint32_t a = (uint32_t)seed, b = (uint32_t)(seed >> 32);
    for (int r = 0; r < 10; ++r) {
        K.k0[r] = a;
        K.k1[r] = b;
        a += kPhW0;
        b += kPhW1;
    }
    return K;
}

// One Philox round, each 32x32 product as its high and low words (mul_hilo).
__device__ __forceinline__ void philox_round(uint32_t& c0, uint32_t& c1, uint32_t& c2, uint32_t& c3, uint32_t k0,
                                             uint32_t k1) {
    uint32_t h0, l0, h1, l1;
    mul_hilo(kPhM0, c0, h0, l0);
    mul_hilo(kPhM1, c2, h1, l1);
    const uint32_t n0 = h1 ^ c1 ^ k0, n2 = h0 ^ c3 ^ k1;
    c1 = l1;
    c3 = l0;
    c0 = n0;
    c2 = n2;
}

// Per-step constant part of a cell draw: the counter words that do not depend on the
// cell (t in word 3, the id's high word 0 in word 2) make the first product of round 1
// and both words of round 2's first product uniform across a sub-step. DrawStep holds
// them; draw_fast() then needs 17 per-cell 32x32 products instead of 19. Valid only for
// ids below 2^32 (lattices of fewer than 4.29e9 cells); the caller checks that.
struct DrawStep {
    uint32_t c0_1, c1_1;    // words 1, 2 after round 1 (uniform)
    uint32_t hi0_2, lo0_2;  // M0 * c0_1 (uniform, used in round 2)
};

__device__ __forceinline__ PhiloxKeys philox_keys_dev(uint64_t seed) { return philox_keys(seed); }

__device__ __forceinline__ DrawStep draw_step(const PhiloxKeys& K, int64_t t) {
    DrawStep s;
    const uint64_t p1 = (uint64_t)kPhM1 * (uint32_t)(uint64_t)t;
    s.c0_1 = (uint32_t)(p1 >> 32) ^ K.k0[0];  // ^ c1, the id's high word, which is 0
    s.c1_1 = (uint32_t)p1;
    const uint64_t p0 = (uint64_t)kPhM0 * s.c0_1;
    s.hi0_2 = (uint32_t)(p0 >> 32);
    s.lo0_2 = (uint32_t)p0;
    return s;
}

// Words 1 and 2 of the draw of cell `id` (< 2^32) with draw index k at the sub-step of s.
__device__ __forceinline__ uint2 draw_fast(const DrawStep& s, const PhiloxKeys& K, uint32_t id, uint32_t k) {
    uint32_t qh, ql;
    mul_hilo(kPhM0, id, qh, ql);  // round 1: c0 = id, c2 = t, c3 = k
    uint32_t c0 = s.c0_1, c1 = s.c1_1, c2 = qh ^ k ^ K.k1[0], c3 = ql;
    {   // round 2: the M0 product of c0 is uniform
        uint32_t h1, l1;
        mul_hilo(kPhM1, c2, h1, l1);
        const uint32_t n0 = h1 ^ c1 ^ K.k0[1], n2 = s.hi0_2 ^ c3 ^ K.k1[1];
        c1 = l1;
        c3 = s.lo0_2;
        c0 = n0;
        c2 = n2;
    }
#pragma unroll
    for (int r = 2; r < 9; ++r) philox_round(c0, c1, c2, c3, K.k0[r], K.k1[r]);
    uint32_t h1, l1;
    mul_hilo(kPhM1, c2, h1, l1);  // round 10: words 1 and 2 only
    return make_uint2(h1 ^ c1 ^ K.k0[9], l1);
}

// ----------------------------------------------------------------- boundaries

// 0-based version of _map_axis (src/spaces.jl:46-51): the mapped index, or -1 when the
// index lies beyond a Constant edge.
__host__ __device__ __forceinline__ int64_t map_axis(int32_t b, int64_t g, int64_t n) {
    if ((uint64_t)g < (uint64_t)n) return g;  // inside: every boundary maps to itself
    if (b == GBCA_PERIODIC) {
        int64_t m = g % n;
        return m < 0 ? m + n : m;
    }
    if (b == GBCA_REFLECTING) {
        int64_t m = g % (2 * n);
        if (m < 0) m += 2 * n;
        return m < n ? m : 2 * n - 1 - m;
    }
    return (g >= 0 && g < n) ? g : -1;
}

// ----------------------------------------------------------------- sweep parameters

// Everything a sweep launch needs besides the buffers. Plain data, passed by value.
struct SweepParams {
    int64_t n1, n2, pitch;     // lattice dims; bytes between consecutive columns
    int32_t bnd[2];
    int32_t cval[2];           // Constant value per axis (as the state's element value)
    int32_t rule, nbhd, radius, states;
    uint64_t birth, survive;
    uint64_t seed;
    int32_t scheme;            // gate kind
    int32_t gate_f32;
    uint64_t gate_thr;         // Stochastic(p) threshold
    uint64_t thr_p, thr_f;     // forest fire thresholds (draws 1 and 2)
    int32_t params_f32;
    int32_t nsub;              // sub-steps in this launch (steps * gates)
    int32_t ngates;            // 2 for Checkerboard, else 1
    int32_t sub0;              // index of the first sub-step within its step (0 or 1)
    int64_t t0;                // time of the first sub-step's step
    int32_t tile_x, tile_y;    // output tile
    int32_t halo_x, halo_y;    // loaded halo (>= nsub * radius)
    PhiloxKeys keys;           // round keys of `seed` (set by the launchers that use them)
    int32_t states_valid;      // every state is known to be one the rule produces (Generations
                               // 0..C-1, forest fire 0..2)
    int32_t staging;           // forest fire: 1 = stage tiles by TMA where the tile fits
    const uint8_t* mask;       // nonzero = the cell updates (pitch bytes between columns), or null
    // active-tile scheduling: the tiles (ty * tiles_x + tx, tiles of tile_x x tile_y cells) to
    // run, *tile_count of them; each run tile writes whether it holds a non-background cell
    const int32_t* tile_list;
    const int32_t* tile_count;
    uint8_t* flags_out;
    int32_t tiles_x;
    int32_t background;
    // the lattice as a slab of a larger one (gbca_set_slab): local column j is global column
    // (j + col0) mod n2g, whose cell ids and Checkerboard parities the sweep uses. col0 = 0 and
    // n2g = n2 for a lattice of its own.
    int64_t col0, n2g;
};

// The global column of mapped local column `my` (0 <= my < n2): one wrap at most, since
// |col0| < n2g and n2 <= n2g.
__host__ __device__ __forceinline__ int64_t global_col(const SweepParams& p, int64_t my) {
    int64_t g = my + p.col0;
    if (g < 0) g += p.n2g;
    else if (g >= p.n2g) g -= p.n2g;
    return g;
}

// Where a lattice lies in a larger one along axis 2 (gbca_set_slab).
struct SlabPlace {
    int64_t col0, n2g;
};

// Active-tile scheduling state of a handle (sweep_sparse.cu): only tiles holding a cell
// other than `background`, and tiles within reach of them, are swept; the others are known
// to stay background (the rule is quiescent).
struct SparseTiles {
    int32_t background;
    int32_t tile_w, tile_h;    // tile size in cells (tile_w a multiple of 32)
    int32_t tiles_x, tiles_y;
    uint8_t* flags[2];         // per state buffer: the tile holds a non-background cell
    int32_t* list;             // candidate tiles of the current pass
    int32_t* count;
};

// The message gbca_last_error() returns on this thread.
void set_last_error(const char* msg);

// Per-device launch facts, looked up once (launch_cache.cu): raise a kernel's dynamic
// shared-memory limit to at least `bytes` (the runtime is called only when the limit set
// before is lower), the SM count, the opt-in shared memory per block, and resident blocks per SM.
cudaError_t ensure_dynamic_smem(const void* fn, size_t bytes);
int device_sms();
int smem_optin();
int blocks_per_sm(const void* fn, int threads, size_t smem);

// Process-wide count of kernel launches (gbca_kernel_launches).
void count_launch(int64_t n = 1);
int64_t launches_so_far();

// Kernel selection and temporally blocked passes for an Int8 problem (sweep_dispatch.cu):
// nsteps steps between bufs[*cur] and bufs[*cur ^ 1], *cur updated.
SweepParams sweep_params(const gbca_desc& d, int64_t pitch, const double* params);
// A kernel geometry choice: steps per temporally blocked pass, tile height (0 = default) and
// how the forest-fire kernel stages its tiles (0 = vector loads, 1 = TMA where it fits).
struct SweepChoice {
    int32_t steps_per_pass;
    int32_t tile_rows;
    int32_t staging;
    int32_t tile_words = 0;  // bit-sliced kernel: tile width in 32-cell words (0: up to 32)
};

// states_valid: every state is known to be one the rule produces (Generations: 0..C-1,
// enabling the bit-sliced kernel; forest fire: 0..2, enabling bit tests on the first step).
// force: use this geometry instead of the autotuner's cached pick (tune.cu).
// mask: cells whose byte is 0 keep their state (general kernel only).
// sparse: sweep only the active tiles (general kernel, tiles of sparse->tile cells).
cudaError_t sweep_int8(const gbca_desc& d, int64_t pitch, int8_t* const bufs[2], int* cur, int64_t t, int64_t nsteps,
                       const double* params, cudaStream_t st, bool states_valid = false,
                       const SweepChoice* force = nullptr, const uint8_t* mask = nullptr,
                       const SparseTiles* sparse = nullptr, const SlabPlace* slab = nullptr);

// Active-tile scheduling (sweep_sparse.cu).
cudaError_t launch_candidates(const SweepParams& p, const SparseTiles& sp, int cur, int halo, cudaStream_t st);
cudaError_t launch_tile_flags(const int8_t* u, int64_t n1, int64_t n2, int64_t pitch, const SparseTiles& sp,
                              uint8_t* flags, cudaStream_t st);
// Whether a background cell whose neighbours are all background stays background.
bool rule_quiescent(const gbca_desc& d, const double* params, int32_t background);

// The geometry the next sweep of a problem uses: the pinned one, the tuned one, or the kernel's
// default (steps per pass filled in for the fast kernels).
SweepChoice sweep_choice(const gbca_desc& d, bool fire, bool life, const SweepChoice* force);

// The autotuner's cached choice for a problem shape (tune.cu); false when it has none.
bool tuned_choice(const gbca_desc& d, SweepChoice* out);
void store_choice(const gbca_desc& d, const SweepChoice& c);
void forget_choices();
// The geometries the autotuner times for a problem (empty: the general kernel, nothing to tune).
std::vector<SweepChoice> sweep_candidates(const SweepParams& p);

// Sub-steps per pass of the general kernel (steps = this / (r x gates), at least 1): the kernel
// is compute-bound (shared-memory neighbour reads, per-cell rule), so deep passes, whose halos
// grow by r per sub-step around a 64 x 64 tile, cost more in recomputed halo than they save in
// HBM traffic.
constexpr int kGenericSubsteps = 4;

// Launchers (one translation unit each).
cudaError_t launch_generic(const SweepParams& p, const int8_t* src, int8_t* dst, cudaStream_t st);
// The general kernel over the tiles of p.tile_list (grid: the number of tiles of the lattice).
cudaError_t launch_generic_tiles(const SweepParams& p, int ntiles, const int8_t* src, int8_t* dst, cudaStream_t st);
bool life_simd_supported(const SweepParams& p);
// The bit-sliced kernel's geometry for a lattice with no tuned or pinned one (sweep_life.cu).
SweepChoice life_default_choice(const SweepParams& p);
cudaError_t launch_life_simd(const SweepParams& p, const int8_t* src, int8_t* dst, cudaStream_t st);
// The bit-sliced kernel over the tiles of p.tile_list (tiles of tile_w x tile_h cells).
cudaError_t launch_life_tiles(const SweepParams& p, const SparseTiles& sp, const int8_t* src, int8_t* dst,
                              cudaStream_t st);
int life_steps_per_pass(const SweepParams& p);
// Whether a pass of `steps` steps on tiles `rows` high fits the bit-sliced kernel's shared memory.
bool life_choice_fits(const SweepParams& p, int steps, int rows);
bool fire_fast_supported(const SweepParams& p);
// A forest-fire sweep with a gate (Stochastic, Checkerboard) or a mask: one sub-step per launch.
bool fire_gated(const SweepParams& p);
// One step of a gated or masked forest fire at time t: a launch per sub-step (Checkerboard's two
// halves in turn), *cur updated after each. Counts its launches.
cudaError_t fire_gated_step(SweepParams& p, int8_t* const bufs[2], int* cur, int64_t t, cudaStream_t st);
// p.tile_y: a pinned tile height, or 0 for the launcher's model.
cudaError_t launch_fire(const SweepParams& p, const int8_t* src, int8_t* dst, cudaStream_t st);

// The forest-fire kernel's output tile (cells along axis 1 x axis 2; the launcher picks the
// height of one-step passes, kFireTileRows is the persistent ensemble pass's).
constexpr int kFireTileCols = 256, kFireTileRows = 128;
constexpr int kFireRowsMin = 8, kFireRowsMax = 240;  // heights gbca_set_geometry accepts for the fire kernel
// Whether tiles of `rows` rows fit shared memory at `steps` steps per pass and that staging.
bool fire_rows_fit(int steps, int rows, int staging);

// One lattice of a batched forest-fire sweep (many lattices per launch, one pass each).
struct FireJob {
    SweepParams p;       // its sweep: t0 = time of its first step; keys and thresholds set
    int8_t* buf[2];      // its two state buffers (pitch p.pitch, 16-byte aligned)
    int64_t nsteps;      // steps of this run
    int32_t cur0;        // buffer holding the state before the first pass
    int32_t tiles_x;     // output tiles along axis 1
    int32_t tile0;       // its first tile in the launch's tile order
    int32_t inst;        // the caller's index of the lattice
};
// Pass `pass` (steps pass*K .. pass*K + K - 1 of every job, fewer where a job ends) over all
// jobs' tiles: block b runs tile b of the concatenated order, tile_job[b] naming its job.
// Jobs whose steps are all done leave their blocks idle. 1 <= K <= 16. Not counted in
// gbca_kernel_launches (the batched ensemble counts its graph's kernels per replay).
cudaError_t launch_fire_batch(const FireJob* jobs, const int32_t* tile_job, int ntiles, int pass, int K,
                              cudaStream_t st);
// Tiles whose TMA copy did not complete within its wait limit since the last call (cleared).
int fire_tma_timeouts_take();
// One bounded wait (`polls` polls) on a barrier nothing completes: exercises the timeout path.
cudaError_t launch_wait_probe(int polls, cudaStream_t st);

}  // namespace gbca
