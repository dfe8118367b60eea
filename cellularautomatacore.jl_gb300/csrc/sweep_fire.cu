// sweep_fire.cu — the forest-fire sweep (Int8 codes 0 empty, 1 tree, 2 fire;
// VonNeumann(1); Synchronous), temporally blocked.
//
// The rule (the package README's LocalRule, restated on Int8):
//   2 -> 0;  0 -> 1 if bernoulli(p, draw 1);  1 -> 2 if a neighbour burns,
//   else 2 if bernoulli(f, draw 2), else 1.
// Each drawing cell costs one Philox4x32-10 evaluation keyed (seed; id, 0, t, k) as
// src/random.jl:102-107, so the kernel is bound by 32x32-bit multiplies, not by HBM.
// draw_fast() hoists the products that do not depend on the cell out of the cell loop,
// and temporal blocking (nsub steps per pass, halo nsub) keeps HBM traffic at
// 2 B / nsub per cell-update.
//
// Tile staging (the autotuner's choice, p.staging: 0 vector loads, 1 a TMA copy per tile, 2 the
// same from a persistent kernel that prefetches each CTA's next tile): where the tile's loaded
// region lies inside
// the lattice, or the lattice is a Grid with Constant(0) edges (the tensor's zero fill is then
// the boundary value), one TMA
// copy (cp.async.bulk.tensor) brings the whole halo-padded tile into shared memory (for the
// zero-fill case n1 must be a multiple of 16, so no box reaches the column padding). The state
// is viewed as a 3-D tensor (16-byte segments x segments x rows), so a box of
// 16 x (sx / 16) x sy lands as rows of sx bytes, the tile's own layout. Other tiles load
// through the boundary map. The copy's completion is awaited on an mbarrier with an
// iteration limit; on expiry the CTA records a timeout (reported by gbca_sync /
// gbca_get_state), waits once more with a limit and leaves its tile unwritten.
#include <cuda.h>

#include <cstring>
#include <mutex>
#include <vector>

#include "fire_words.cuh"
#include "gbca_internal.cuh"

namespace gbca {

__device__ int g_fire_tma_timeouts = 0;

namespace {

constexpr int kFireTX = kFireTileCols, kFireTY = kFireTileRows;
constexpr int kFireThreadsX = 32, kFireThreadsY = 16;
// k_fire (one-step passes over at least as many tiles as SMs) and the batched kernel run
// 256-thread CTAs, four an SM within 64 registers (a one-step pass keeps one shared buffer, 46 KB
// for 158-row tiles), against two 512-thread CTAs before: smaller CTAs fill the SMs more evenly
// (ensemble of 4096 instances 294.9 -> 311.2 Gcell-updates/s; 4096^2 fire 304 -> 329, 16384^2
// 387 -> 408 on a box where the wider form ran slower). Deeper passes and lattices of fewer tiles
// than SMs keep 512-thread CTAs: each tile's work spread over more threads. k_fire_stream keeps
// 512 threads.
constexpr int kFireBatchThreadsY = 8, kFireTileThreadsY = 8;
constexpr int kFireRowsOneStep = 160;  // the tallest tile the one-step model considers
constexpr int kFireTileCost = 16;      // a tile's fixed cost in rows (see launch_fire)
constexpr int kTmaSpins = 1 << 22;  // try_wait polls before a tile gives up

__device__ __forceinline__ uint32_t smem_u32(const void* p) { return (uint32_t)__cvta_generic_to_shared(p); }

__device__ __forceinline__ bool mbar_try_wait(uint64_t* bar, uint32_t phase) {
    uint32_t ok;
    asm volatile(
        "{\n\t.reg .pred p;\n\t"
        "mbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\n\t"
        "selp.u32 %0, 1, 0, p;\n\t}"
        : "=r"(ok)
        : "r"(smem_u32(bar)), "r"(phase)
        : "memory");
    return ok != 0;
}

__device__ __forceinline__ bool mbar_wait_bounded(uint64_t* bar, uint32_t phase, int limit = kTmaSpins) {
    for (int it = 0; it < limit; ++it)
        if (mbar_try_wait(bar, phase)) return true;
    return false;
}

// The timeout path on purpose: one bounded wait on a barrier that nothing completes (no copy is
// issued), recorded like a tile copy that gave up. Nothing is in flight when the CTA leaves.
__global__ void k_wait_probe(int polls) {
    __shared__ __align__(8) uint64_t bar;
    if (threadIdx.x == 0) {
        asm volatile("mbarrier.init.shared::cta.b64 [%0], 1;" ::"r"(smem_u32(&bar)) : "memory");
        asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
    }
    __syncthreads();
    const bool ok = __syncthreads_and(mbar_wait_bounded(&bar, 0, polls));
    if (!ok && threadIdx.x == 0) atomicAdd(&g_fire_tma_timeouts, 1);
}

// One thread: arm the barrier for `bytes` and issue the 3-D tile copy into `dst`.
__device__ __forceinline__ void tma_tile_load(const CUtensorMap* map, void* dst, uint64_t* bar, int seg0, int row0,
                                              uint32_t bytes) {
    asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;" ::"r"(smem_u32(bar)), "r"(bytes)
                 : "memory");
    asm volatile(
        "cp.async.bulk.tensor.3d.shared::cluster.global.tile.mbarrier::complete_tx::bytes [%0], [%1, {%2, %3, %4}], "
        "[%5];" ::"r"(smem_u32(dst)),
        "l"((uint64_t)map), "r"(0), "r"(seg0), "r"(row0), "r"(smem_u32(bar))
        : "memory");
}

// The halo-padded region of a tile that reaches past the lattice's edges: sx x sy bytes from
// lattice (X0 - hx, Y0 - hy) through the boundary map (a row beyond a Constant edge of axis 2
// holds its constant; else a cell beyond a Constant edge of axis 1 holds that constant). First
// by 16-byte segments (X0 - hx, sx and the pitch are multiples of 16): a segment inside the
// lattice's columns is one vector load, a row or segment wholly beyond a Constant edge one
// vector fill. The remaining columns — a segment straddling column n1, or beyond a Periodic or
// Reflecting edge — then map byte by byte, one byte per thread, so no warp waits on a few
// lanes' byte loops.
__device__ __forceinline__ void load_region_mapped(const SweepParams& p, const int8_t* __restrict__ src, int8_t* A,
                                                   int64_t X0, int64_t Y0, int hx, int hy, int sx, int sy, int tid,
                                                   int nthr) {
    const int qx = sx / 16;
    const int64_t gx0 = X0 - hx;
    const bool cst0 = p.bnd[0] == GBCA_CONSTANT;
    const uint32_t c0 = (uint32_t)(uint8_t)p.cval[0] * 0x01010101u, c1 = (uint32_t)(uint8_t)p.cval[1] * 0x01010101u;
    for (int q = tid; q < qx * sy; q += nthr) {
        const int lq = q % qx, ly = q / qx;
        const int64_t gx = gx0 + 16 * lq;
        const int64_t my = map_axis(p.bnd[1], Y0 - hy + ly, p.n2);
        int4* out = (int4*)(A + ly * sx + 16 * lq);
        if (my < 0) {
            *out = make_int4((int)c1, (int)c1, (int)c1, (int)c1);
        } else if (gx >= 0 && gx + 16 <= p.n1) {
            *out = *(const int4*)(src + gx + my * p.pitch);
        } else if (cst0 && (gx + 16 <= 0 || gx >= p.n1)) {
            *out = make_int4((int)c0, (int)c0, (int)c0, (int)c0);
        }
    }
    // the byte-mapped columns: [0, nl) before the lattice (beyond a Periodic or Reflecting
    // edge), and [r0, r1) from the first segment not wholly inside it: with a Constant axis 1
    // the straddling segment only (the ones beyond were filled above), else every column on
    const int nl = (!cst0 && gx0 < 0) ? (int)(-gx0 < (int64_t)sx ? -gx0 : (int64_t)sx) : 0;
    const int64_t a = p.n1 - gx0;  // region columns from its left edge to column n1 (> 0)
    int r0 = sx, r1 = sx;
    if (a < sx) {
        r0 = (int)(a / 16 * 16);
        r1 = cst0 ? (a % 16 ? r0 + 16 : r0) : sx;
    }
    const int ncols = nl + (r1 - r0);
    if (ncols == 0) return;
    for (int idx = tid; idx < ncols * sy; idx += nthr) {
        const int k = idx % ncols, ly = idx / ncols;
        const int lx = k < nl ? k : r0 + (k - nl);
        const int64_t my = map_axis(p.bnd[1], Y0 - hy + ly, p.n2);
        if (my < 0) continue;  // the row's constant is already in place
        const int64_t mx = map_axis(p.bnd[0], gx0 + lx, p.n1);
        A[ly * sx + lx] = mx < 0 ? (int8_t)p.cval[0] : src[mx + my * p.pitch];
    }
}

// Four cells (one 32-bit word of the shared tile) per work item: neighbour tests in byte
// SIMD, then four independent Philox chains.
template <bool INTERIOR, bool GATED, int ROWS>
__device__ __forceinline__ void fire_tile(const SweepParams& p, const int8_t* __restrict__ src,
                                          int8_t* __restrict__ dst, int8_t* A, int8_t* B, bool staged,
                                          int64_t X0, int64_t Y0) {
    const int hx = p.halo_x, hy = p.halo_y;
    const int TY = p.tile_y;  // the tile's rows (the launcher's choice)
    const int sx = kFireTX + 2 * hx, sy = TY + 2 * hy;
    const int sw = sx / 4;  // words per shared row
    const int tid = threadIdx.y * kFireThreadsX + threadIdx.x;
    const int nthr = kFireThreadsX * blockDim.y;  // 8 rows of threads (16 in k_fire_stream)

    if (staged) {  // the tile arrived by TMA
    } else if (INTERIOR) {  // 16-byte loads: X0 - hx, sx and the pitch are multiples of 16
        const int qx = sx / 16;
        for (int q = tid; q < qx * sy; q += nthr) {
            const int lq = q % qx, ly = q / qx;
            const int4 v = *(const int4*)(src + (X0 - hx + 16 * lq) + (Y0 - hy + ly) * p.pitch);
            *(int4*)(A + ly * sx + 16 * lq) = v;
        }
    } else {
        load_region_mapped(p, src, A, X0, Y0, hx, hy, sx, sy, tid, nthr);
    }
    __syncthreads();

    FireGeom g;
    g.n1 = p.n1;
    g.n2 = p.n2;
    g.bnd0 = p.bnd[0];
    g.bnd1 = p.bnd[1];
    g.cst0 = (uint32_t)(uint8_t)p.cval[0] * 0x01010101u;
    g.cst1 = (uint32_t)(uint8_t)p.cval[1] * 0x01010101u;
    fire_thresholds(p.thr_p, p.thr_f, p.params_f32 != 0, g);
    g.exact_always = fire_odd_constant(p.bnd[0], p.cval[0], p.bnd[1], p.cval[1]);
    g.col0 = p.col0;
    g.n2g = p.n2g;
    for (int s = 0; s < p.nsub; ++s) {
        const DrawStep ds = draw_step(p.keys, p.t0 + s);
        const int ex = p.nsub - 1 - s;
        const int w_lo = (hx - ex) >> 2, w_hi = (hx + kFireTX + ex + 3) >> 2;  // words covering the region
        const bool exact = s == 0 && !p.states_valid;
        if (p.nsub == 1) {
            // one step: the region is the tile itself (64 words, all 512 threads busy walking
            // rows), stored straight to the lattice state; a ragged last tile spreads the
            // threads over the words and rows inside the lattice only
            int nw = kFireTX / 4, nrows = TY;
            if (!INTERIOR) {
                if (p.n1 - X0 < kFireTX) nw = (int)((p.n1 - X0 + 3) / 4);
                if (p.n2 - Y0 < TY) nrows = (int)(p.n2 - Y0);
            }
            FireGate fg;  // a gated or masked sweep runs one sub-step per launch, half p.sub0
            if constexpr (GATED) fire_gate(p.scheme, p.sub0 % p.ngates, p.gate_thr, p.gate_f32, p.mask, p.pitch, fg);
            fire_substep_rows<!INTERIOR, GATED, ROWS>((const uint32_t*)A, sw, hx >> 2, nw, hy, nrows, X0 - hx,
                                                      Y0 - hy, g, ds, p.keys, tid, nthr, exact, dst, p.pitch, &fg);
            return;
        }
        // deeper passes: the region is wider than the tile in early sub-steps, so the flat
        // word x row split keeps every thread busy
        fire_substep_words<!INTERIOR>((const uint32_t*)A, (uint32_t*)B, sw, w_lo, w_hi - w_lo, hy - ex,
                                      TY + 2 * ex, X0 - hx, Y0 - hy, g, ds, p.keys, tid, nthr, exact);
        __syncthreads();
        int8_t* t = A; A = B; B = t;
    }

    if (INTERIOR) {  // 16-byte stores: X0, the tile width and the pitch are multiples of 16
        const int qx = kFireTX / 16;
        for (int q = tid; q < qx * TY; q += nthr) {
            const int lq = q % qx, oy = q / qx;
            *(int4*)(dst + (X0 + 16 * lq) + (Y0 + oy) * p.pitch) = *(const int4*)(A + (hy + oy) * sx + hx + 16 * lq);
        }
    } else {
        for (int idx = tid; idx < kFireTX * TY; idx += nthr) {
            const int ox = idx % kFireTX, oy = idx / kFireTX;
            const int64_t gx = X0 + ox, gy = Y0 + oy;
            if (gx < p.n1 && gy < p.n2) dst[gx + gy * p.pitch] = A[(hy + oy) * sx + hx + ox];
        }
    }
}

// tma: 0 = no tensor map; 1 = stage interior tiles by TMA; 2 = every tile (Constant(0) edges).
// GATED: a one-step sweep with a gate or a mask (compiled apart, so the synchronous kernel keeps
// its registers).
template <bool GATED, bool WIDE>
__global__ void __launch_bounds__(kFireThreadsX*(WIDE ? kFireThreadsY : kFireTileThreadsY), WIDE ? 1 : 4)
    k_fire(SweepParams p, const int8_t* __restrict__ src, int8_t* __restrict__ dst,
           const __grid_constant__ CUtensorMap tmap, int tma) {
    extern __shared__ __align__(128) int8_t smem_f[];
    __shared__ __align__(8) uint64_t tma_bar;
    const int sx = kFireTX + 2 * p.halo_x, sy = p.tile_y + 2 * p.halo_y;
    int8_t* A = smem_f;
    int8_t* B = smem_f + sx * sy;
    const int64_t X0 = (int64_t)blockIdx.x * kFireTX, Y0 = (int64_t)blockIdx.y * p.tile_y;
    const bool interior = X0 - p.halo_x >= 0 && X0 + kFireTX + p.halo_x <= p.n1 && Y0 - p.halo_y >= 0 &&
                          Y0 + p.tile_y + p.halo_y <= p.n2;
    // a tensor copy's shared destination must be 128-byte aligned (the dynamic base is)
    const bool staged = (smem_u32(A) & 127u) == 0u && (tma == 2 || (tma == 1 && interior));
    if (staged) {
        const int tid = threadIdx.y * kFireThreadsX + threadIdx.x;
        if (tid == 0) {
            asm volatile("mbarrier.init.shared::cta.b64 [%0], 1;" ::"r"(smem_u32(&tma_bar)) : "memory");
            asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
            asm volatile("fence.proxy.async.shared::cta;" ::: "memory");
        }
        __syncthreads();
        // the region starts at lattice (X0 - halo_x, Y0 - halo_y): segment (X0 - halo_x) / 16,
        // a whole number since X0 and halo_x are multiples of 16; innermost coordinate 0
        if (tid == 0)
            tma_tile_load(&tmap, A, &tma_bar, (int)((X0 - p.halo_x) / 16), (int)(Y0 - p.halo_y),
                          (uint32_t)(sx * sy));
        const bool ok = __syncthreads_and(mbar_wait_bounded(&tma_bar, 0));
        if (!ok) {
            if (tid == 0) atomicAdd(&g_fire_tma_timeouts, 1);
            mbar_wait_bounded(&tma_bar, 0);  // let a late copy land before the CTA leaves
            return;
        }
    }
    // two rows of the walk unrolled together; the gated form keeps one (its registers)
    if (interior) fire_tile<true, GATED, GATED ? 1 : 2>(p, src, dst, A, B, staged, X0, Y0);
    else fire_tile<false, GATED, GATED ? 1 : 2>(p, src, dst, A, B, staged, X0, Y0);
}

// Many lattices per launch (a batched ensemble's large instances): one pass of up to K steps
// over every tile of every job, block b running tile b of the concatenated tile order. Pass q
// of a job reads buffer cur0 ^ (q & 1) and writes the other, so a job's passes ping-pong as a
// single lattice's do; a job with no steps left at pass q leaves its blocks idle. Tiles load
// with 16-byte vector loads inside the lattice and through the boundary map at its edges.
__global__ void __launch_bounds__(kFireThreadsX* kFireBatchThreadsY, 4)
    k_fire_batch(const FireJob* __restrict__ jobs, const int32_t* __restrict__ tile_job, int pass, int K) {
    extern __shared__ __align__(128) int8_t smem_f[];
    __shared__ SweepParams sp;
    const FireJob& J = jobs[tile_job[blockIdx.x]];
    const int64_t done = (int64_t)pass * K;
    if (done >= J.nsteps) return;  // the whole block: the job ended in an earlier pass
    const int nsub = (int)(J.nsteps - done < K ? J.nsteps - done : K);
    const int tid = threadIdx.y * kFireThreadsX + threadIdx.x;
    for (int k = tid; k < (int)(sizeof(SweepParams) / 4); k += kFireThreadsX * kFireBatchThreadsY)
        ((uint32_t*)&sp)[k] = ((const uint32_t*)&J.p)[k];
    __syncthreads();
    if (tid == 0) {
        sp.tile_y = kFireTY;
        sp.nsub = nsub;
        sp.t0 = J.p.t0 + done;
        sp.halo_y = nsub;
        sp.halo_x = (nsub + 15) / 16 * 16;
        if (pass > 0) sp.states_valid = 1;  // a pass leaves only 0, 1 and 2
    }
    __syncthreads();
    const int local = (int)blockIdx.x - J.tile0;
    const int64_t X0 = (int64_t)(local % J.tiles_x) * kFireTX, Y0 = (int64_t)(local / J.tiles_x) * kFireTY;
    const int c = J.cur0 ^ (pass & 1);
    const int8_t* src = J.buf[c];
    int8_t* dst = J.buf[c ^ 1];
    const int sx = kFireTX + 2 * sp.halo_x, sy = kFireTY + 2 * sp.halo_y;
    int8_t* A = smem_f;
    int8_t* B = smem_f + sx * sy;
    const bool interior = X0 - sp.halo_x >= 0 && X0 + kFireTX + sp.halo_x <= sp.n1 && Y0 - sp.halo_y >= 0 &&
                          Y0 + kFireTY + sp.halo_y <= sp.n2;
    if (interior) fire_tile<true, false, 1>(sp, src, dst, A, B, false, X0, Y0);
    else fire_tile<false, false, 1>(sp, src, dst, A, B, false, X0, Y0);
}

// One step per pass with TMA staging, persistent: each CTA walks the tiles blockIdx.x,
// blockIdx.x + gridDim.x, ... While it computes one tile from one shared buffer, the TMA copy
// of its next tile fills the other, so the copy's latency hides behind the Philox work; the
// last (only) sub-step stores straight to HBM, so no third buffer is needed. Tiles that TMA
// cannot stage (beyond an edge that is not Constant(0)) load through the boundary map.
template <bool GATED>
__global__ void __launch_bounds__(kFireThreadsX* kFireThreadsY)
    k_fire_stream(SweepParams p, const int8_t* __restrict__ src, int8_t* __restrict__ dst,
                  const __grid_constant__ CUtensorMap tmap, int tma, int tiles_x, int ntiles) {
    extern __shared__ __align__(128) int8_t smem_f[];
    __shared__ __align__(8) uint64_t bars[2];
    const int hx = p.halo_x, hy = p.halo_y;  // halo_y = 1: one step per pass
    const int TY = p.tile_y;                   // the tile's rows (the launcher's choice)
    const int sx = kFireTX + 2 * hx, sy = TY + 2 * hy, sw = sx / 4;
    // a tensor copy's shared destination must be 128-byte aligned: buffers start on 128 bytes
    const int stride = (sx * sy + 127) / 128 * 128;
    int8_t* const buf0 = smem_f;
    int8_t* const buf1 = smem_f + stride;
    const bool aligned = ((smem_u32(buf0) | smem_u32(buf1)) & 127u) == 0u;
    const int tid = threadIdx.y * kFireThreadsX + threadIdx.x;
    const int nthr = kFireThreadsX * kFireThreadsY;
    FireGeom g;
    g.n1 = p.n1;
    g.n2 = p.n2;
    g.bnd0 = p.bnd[0];
    g.bnd1 = p.bnd[1];
    g.cst0 = (uint32_t)(uint8_t)p.cval[0] * 0x01010101u;
    g.cst1 = (uint32_t)(uint8_t)p.cval[1] * 0x01010101u;
    fire_thresholds(p.thr_p, p.thr_f, p.params_f32 != 0, g);
    g.exact_always = fire_odd_constant(p.bnd[0], p.cval[0], p.bnd[1], p.cval[1]);
    g.col0 = p.col0;
    g.n2g = p.n2g;
    const DrawStep ds = draw_step(p.keys, p.t0);
    FireGate fg;  // a gated or masked sweep: one sub-step, half p.sub0
    if constexpr (GATED) fire_gate(p.scheme, p.sub0 % p.ngates, p.gate_thr, p.gate_f32, p.mask, p.pitch, fg);
    if (tid == 0) {
        asm volatile("mbarrier.init.shared::cta.b64 [%0], 1;" ::"r"(smem_u32(&bars[0])) : "memory");
        asm volatile("mbarrier.init.shared::cta.b64 [%0], 1;" ::"r"(smem_u32(&bars[1])) : "memory");
        asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
        asm volatile("fence.proxy.async.shared::cta;" ::: "memory");
    }
    __syncthreads();
    auto origin = [&](int tile, int64_t* X0, int64_t* Y0) {
        *X0 = (int64_t)(tile % tiles_x) * kFireTX;
        *Y0 = (int64_t)(tile / tiles_x) * TY;
        return *X0 - hx >= 0 && *X0 + kFireTX + hx <= p.n1 && *Y0 - hy >= 0 && *Y0 + TY + hy <= p.n2;
    };
    auto staged = [&](bool interior) { return aligned && (tma == 2 || (tma == 1 && interior)); };
    auto issue = [&](int tile, int k) {  // one thread: the tile's copy into buffer k
        int64_t X0, Y0;
        origin(tile, &X0, &Y0);
        // order the buffer's earlier generic-proxy reads and writes (finished at the last
        // barrier) before the async-proxy copy that overwrites it
        asm volatile("fence.proxy.async.shared::cta;" ::: "memory");
        tma_tile_load(&tmap, k ? buf1 : buf0, &bars[k], (int)((X0 - hx) / 16), (int)(Y0 - hy), (uint32_t)(sx * sy));
    };
    uint32_t phase = 0u;  // bit k: the parity buffer k's barrier completes next
    uint32_t pend = 0u;   // bit k: a copy was issued into buffer k and not yet awaited
    int tile = blockIdx.x, b = 0;
    if (tile < ntiles) {
        int64_t X0, Y0;
        if (staged(origin(tile, &X0, &Y0))) {
            if (tid == 0) issue(tile, 0);
            pend |= 1u;
        }
    }
    bool failed = false;
    for (; tile < ntiles; tile += gridDim.x, b ^= 1) {
        const int next = tile + (int)gridDim.x;
        if (next < ntiles) {  // buffer b ^ 1 was last read before the previous iteration's barrier
            int64_t X1, Y1;
            if (staged(origin(next, &X1, &Y1))) {
                if (tid == 0) issue(next, b ^ 1);
                pend |= 1u << (b ^ 1);
            }
        }
        int64_t X0, Y0;
        const bool interior = origin(tile, &X0, &Y0);
        int8_t* const cur = b ? buf1 : buf0;
        if ((pend >> b) & 1u) {
            const bool ok = __syncthreads_and(mbar_wait_bounded(&bars[b], (phase >> b) & 1u));
            phase ^= 1u << b;
            pend &= ~(1u << b);
            if (!ok) {
                failed = true;
                break;
            }
        } else {  // beyond an edge TMA cannot reproduce: the boundary map
            load_region_mapped(p, src, cur, X0, Y0, hx, hy, sx, sy, tid, nthr);
            __syncthreads();
        }
        const uint32_t* A = (const uint32_t*)cur;
        if (interior) {
            fire_substep_rows<false, GATED>(A, sw, hx >> 2, kFireTX / 4, hy, TY, X0 - hx, Y0 - hy, g, ds, p.keys,
                                            tid, nthr, !p.states_valid, dst, p.pitch, &fg);
        } else {  // a ragged last tile: the words and rows inside the lattice only
            const int nw = p.n1 - X0 < kFireTX ? (int)((p.n1 - X0 + 3) / 4) : kFireTX / 4;
            const int nrows = p.n2 - Y0 < TY ? (int)(p.n2 - Y0) : TY;
            fire_substep_rows<true, GATED>(A, sw, hx >> 2, nw, hy, nrows, X0 - hx, Y0 - hy, g, ds, p.keys, tid, nthr,
                                           !p.states_valid, dst, p.pitch, &fg);
        }
        __syncthreads();
    }
    if (failed) {
        if (tid == 0) atomicAdd(&g_fire_tma_timeouts, 1);
        // let the copies in flight land before the CTA leaves: the one that timed out
        // (its parity was flipped above) and a prefetch still pending
        mbar_wait_bounded(&bars[b], ((phase >> b) & 1u) ^ 1u);
        if ((pend >> (b ^ 1)) & 1u) mbar_wait_bounded(&bars[b ^ 1], (phase >> (b ^ 1)) & 1u);
    }
}

// Tensor maps of the state buffers, by buffer and box height (the pass depth sets it).
struct MapKey {
    const void* base;
    int64_t n1, n2, pitch;
    int sx, sy;
};
struct MapEntry {
    MapKey k;
    CUtensorMap map;
};

typedef CUresult (*EncodeTiled)(CUtensorMap*, CUtensorMapDataType, cuuint32_t, void*, const cuuint64_t*,
                                const cuuint64_t*, const cuuint32_t*, const cuuint32_t*, CUtensorMapInterleave,
                                CUtensorMapSwizzle, CUtensorMapL2promotion, CUtensorMapFloatOOBfill);

std::mutex g_map_mu;
// two buffers x the depths and tile heights in use, per lattice: 128 entries cover a server's
// lanes (16 lattices at a time) without one lane evicting another's maps
constexpr size_t kMaxMaps = 128;
std::vector<MapEntry> g_maps;
EncodeTiled g_encode = nullptr;
bool g_encode_looked = false;

// The 3-D view (16-byte segments, segment index, row) of a state buffer with a box of one
// whole tile; false when the driver offers no tensor maps.
bool tile_map(const void* base, int64_t n1, int64_t n2, int64_t pitch, int sx, int sy, CUtensorMap* out) {
    std::lock_guard<std::mutex> lock(g_map_mu);
    for (auto it = g_maps.rbegin(); it != g_maps.rend(); ++it) {  // the most recent first
        const MapEntry& m = *it;
        if (m.k.base == base && m.k.n1 == n1 && m.k.n2 == n2 && m.k.pitch == pitch && m.k.sx == sx && m.k.sy == sy) {
            *out = m.map;
            return true;
        }
    }
    if (!g_encode_looked) {
        g_encode_looked = true;
        void* fn = nullptr;
        cudaDriverEntryPointQueryResult q;
        if (cudaGetDriverEntryPointByVersion("cuTensorMapEncodeTiled", &fn, 12000, cudaEnableDefault, &q) ==
                cudaSuccess &&
            q == cudaDriverEntryPointSuccess)
            g_encode = (EncodeTiled)fn;
        cudaGetLastError();
    }
    if (!g_encode) return false;
    const cuuint64_t dims[3] = {16, (cuuint64_t)((n1 + 15) / 16), (cuuint64_t)n2};
    const cuuint64_t strides[2] = {16, (cuuint64_t)pitch};
    const cuuint32_t box[3] = {16, (cuuint32_t)(sx / 16), (cuuint32_t)sy};
    const cuuint32_t estr[3] = {1, 1, 1};
    CUtensorMap m;
    if (g_encode(&m, CU_TENSOR_MAP_DATA_TYPE_UINT8, 3, const_cast<void*>(base), dims, strides, box, estr,
                 CU_TENSOR_MAP_INTERLEAVE_NONE, CU_TENSOR_MAP_SWIZZLE_NONE, CU_TENSOR_MAP_L2_PROMOTION_L2_128B,
                 CU_TENSOR_MAP_FLOAT_OOB_FILL_NONE) != CUDA_SUCCESS)
        return false;
    if (g_maps.size() >= kMaxMaps) g_maps.erase(g_maps.begin());
    g_maps.push_back(MapEntry{MapKey{base, n1, n2, pitch, sx, sy}, m});
    *out = m;
    return true;
}

}  // namespace

cudaError_t launch_wait_probe(int polls, cudaStream_t st) {
    k_wait_probe<<<1, 32, 0, st>>>(polls);
    count_launch();
    return cudaGetLastError();
}

int fire_tma_timeouts_take() {
    int n = 0;
    if (cudaMemcpyFromSymbol(&n, g_fire_tma_timeouts, sizeof n) != cudaSuccess) {
        cudaGetLastError();
        return 0;
    }
    if (n) {
        const int zero = 0;
        cudaMemcpyToSymbol(g_fire_tma_timeouts, &zero, sizeof zero);
    }
    return n;
}

cudaError_t launch_fire_batch(const FireJob* jobs, const int32_t* tile_job, int ntiles, int pass, int K,
                              cudaStream_t st) {
    if (K < 1 || K > 16 || ntiles < 1) return cudaErrorInvalidValue;
    const int hx = (K + 15) / 16 * 16;
    const size_t smem = 2 * (size_t)(kFireTX + 2 * hx) * (size_t)(kFireTY + 2 * K);
    cudaError_t e = ensure_dynamic_smem((const void*)k_fire_batch, smem);
    if (e != cudaSuccess) return e;
    k_fire_batch<<<ntiles, dim3(kFireThreadsX, kFireBatchThreadsY), smem, st>>>(jobs, tile_job, pass, K);
    return cudaGetLastError();
}

bool fire_fast_supported(const SweepParams& p) {
    // every scheme and masks: a gated or masked sweep runs one sub-step per launch (fire_gated)
    return p.rule == GBCA_RULE_FOREST_FIRE && p.nbhd == GBCA_VON_NEUMANN && p.radius == 1 &&
           (p.scheme == GBCA_SYNCHRONOUS || p.scheme == GBCA_STOCHASTIC || p.scheme == GBCA_CHECKERBOARD) &&
           p.n1 * p.n2g < ((int64_t)1 << 32) - 1 && p.pitch % 16 == 0;
}

bool fire_gated(const SweepParams& p) { return p.scheme != GBCA_SYNCHRONOUS || p.mask != nullptr; }

bool fire_rows_fit(int steps, int rows, int staging) {
    if (rows < kFireRowsMin || rows > kFireRowsMax || steps < 1) return false;
    const int optin = smem_optin();
    const size_t sx = kFireTX + 2 * (size_t)((steps + 15) / 16 * 16), sy = (size_t)rows + 2 * (size_t)steps;
    const size_t smem = staging == 2 && steps == 1 ? 2 * ((sx * sy + 127) / 128 * 128) : 2 * sx * sy;
    return smem <= (size_t)optin;
}

cudaError_t launch_fire(const SweepParams& p0, const int8_t* src, int8_t* dst, cudaStream_t st) {
    SweepParams p = p0;
    p.tile_x = kFireTX;
    // tile rows: pinned, or a model's pick
    if (p0.tile_y > 0) {  // pinned (gbca_set_geometry checked that it fits)
        p.tile_y = p0.tile_y;
    } else if (p.nsub == 1) {
        // one step per pass, any height of 32..160 rows: minimise the busiest SM's tiles,
        // ceil(tiles / SMs), times the cost of a tile, its rows plus kFireTileCost rows' worth
        // of halo, staging and set-up. The constant is fitted to Gcell-updates/s measured by
        // height on 2048^2, 4096^2 and 8192^2 grids; the model's picks there (108, 147 and 158
        // rows) ran fastest of the heights measured, 255, 336 and 387 against 227, 292 and 376
        // for the best of 128, 64 and 32 rows.
        const int64_t tx = (p.n1 + kFireTX - 1) / kFireTX, nsm = device_sms();
        int64_t best = -1;
        for (int ty = kFireRowsOneStep; ty >= 32; --ty) {
            const int64_t t = tx * ((p.n2 + ty - 1) / ty);
            const int64_t cost = (t + nsm - 1) / nsm * (ty + kFireTileCost);
            if (best < 0 || cost < best) {
                best = cost;
                p.tile_y = ty;
            }
        }
    } else {
        // deeper passes: 128, 64 or 32 rows, whichever keeps the most of the GPU busy. The
        // tiles run in rounds of one per CTA slot (two CTAs per SM), so a lattice of t tiles
        // fills (t / slots) / ceil(t / slots) of the last round's share; a shorter tile
        // recomputes a larger share of halo rows, TY / (TY + 2 halo) useful.
        const int64_t tx = (p.n1 + kFireTX - 1) / kFireTX, slots = 2 * (int64_t)device_sms();
        double best = -1.0;
        for (int ty = kFireTY; ty >= 32; ty /= 2) {
            const int64_t t = tx * ((p.n2 + ty - 1) / ty);
            const double rounds = (double)((t + slots - 1) / slots);
            const double eff = ((double)t / (double)slots) / rounds * (double)ty / (double)(ty + 2 * p.nsub);
            if (eff > best + 1e-9) {
                best = eff;
                p.tile_y = ty;
            }
        }
    }
    p.halo_y = p.nsub;
    p.halo_x = (p.nsub + 15) / 16 * 16;
    p.keys = philox_keys(p.seed);
    const int sx = kFireTX + 2 * p.halo_x, sy = p.tile_y + 2 * p.halo_y;
    const int tiles_x = (int)((p.n1 + kFireTX - 1) / kFireTX), tiles_y = (int)((p.n2 + p.tile_y - 1) / p.tile_y);
    // one-step passes over at least as many tiles as SMs: 256-thread CTAs, four an SM, one
    // shared buffer; deeper passes (two buffers) and fewer tiles: 512-thread CTAs
    const bool wide = p.nsub > 1 || (int64_t)tiles_x * tiles_y < device_sms();
    const size_t smem = (wide ? 2 : 1) * (size_t)sx * (size_t)sy;
    const bool gated = fire_gated(p);  // one sub-step per launch (p.nsub == 1), compiled apart
    auto* fire_fn = gated ? (wide ? k_fire<true, true> : k_fire<true, false>)
                          : (wide ? k_fire<false, true> : k_fire<false, false>);
    auto* stream_fn = gated ? k_fire_stream<true> : k_fire_stream<false>;
    cudaError_t e = ensure_dynamic_smem((const void*)fire_fn, smem);
    if (e != cudaSuccess) return e;
    // TMA staging: interior tiles always; every tile when both edges are Constant(0), whose
    // value the tensor's zero fill reproduces, and n1 is a whole number of 16-byte segments
    // (so no box reads the column padding past n1)
    CUtensorMap map;
    std::memset(&map, 0, sizeof map);
    int tma = 0;
    if (p.staging && sy <= 256 && sx / 16 <= 256 && ((uintptr_t)src & 15u) == 0 &&
        tile_map(src, p.n1, p.n2, p.pitch, sx, sy, &map)) {
        const bool zero_edges = p.bnd[0] == GBCA_CONSTANT && p.bnd[1] == GBCA_CONSTANT && p.cval[0] == 0 &&
                                p.cval[1] == 0 && p.n1 % 16 == 0;
        tma = zero_edges ? 2 : 1;
    }
    if (p.nsub == 1 && tma && p.staging == 2) {  // one step per pass: the persistent, double-buffered kernel
        const size_t smem2 = 2 * (((size_t)sx * sy + 127) / 128 * 128);  // two 128-byte-aligned buffers
        e = ensure_dynamic_smem((const void*)stream_fn, smem2);
        if (e != cudaSuccess) return e;
        const int ntiles = tiles_x * tiles_y;
        int grid = device_sms() * blocks_per_sm((const void*)stream_fn, kFireThreadsX * kFireThreadsY, smem2);
        if (grid > ntiles) grid = ntiles;
        stream_fn<<<grid, dim3(kFireThreadsX, kFireThreadsY), smem2, st>>>(p, src, dst, map, tma, tiles_x, ntiles);
        return cudaGetLastError();
    }
    dim3 grid((unsigned)tiles_x, (unsigned)tiles_y);
    fire_fn<<<grid, dim3(kFireThreadsX, wide ? kFireThreadsY : kFireTileThreadsY), smem, st>>>(p, src, dst, map, tma);
    return cudaGetLastError();
}

}  // namespace gbca
