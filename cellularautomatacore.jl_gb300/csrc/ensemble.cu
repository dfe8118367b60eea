// ensemble.cu — batched ensembles: many Int8 problems of different sizes, rules and
// parameters advanced together by ONE persistent kernel launch, captured in a CUDA graph.
//
// This replaces solving an EnsembleProblem trajectory by trajectory (src/problem.jl:571-589,
// SciMLBase's EnsembleSerial / EnsembleThreads; src/calibration.jl:66-91 for ABC), where
// every trajectory allocates, uploads and launches per step on its own.
//
// Scheduling: the host sorts the instances by work (cells x steps), largest first; each CTA
// of a grid sized to fill the GPU pulls the next instance from an atomic counter and runs
// it to the end alone, so no CTA ever waits for another (no inter-CTA barrier, no spin).
// Largest-first keeps the tail short.
//
// Per instance, in one CTA:
//  * small lattices, (n1 + 2r)(n2 + 2r) <= (tile + 16)^2 bytes, live entirely in shared memory: a
//    halo of r cells is refreshed from the boundary map before every step (the halo fill of
//    src/backends.jl:425-442) and all steps run without touching global memory;
//  * larger ones are swept tile by tile with temporal blocking (K steps per pass, halo K r),
//    ping-ponging between the instance's two buffers in global memory (mostly L2-resident).
// At the end the CTA reduces the final state to the exact integers behind state_counts and
// Moran's I (src/measures.jl:14-20,91-107) — the same sums, hence the same bits, as
// gbca_summaries on a single handle.
//
// Large forest-fire instances (2^18 cells or more by default) would each hold one CTA for far
// longer than the rest of the ensemble takes. They run instead as batched multi-lattice passes
// (launch_fire_batch: every tile of every large instance in one launch, one launch per pass of
// K steps) on a second stream forked off the same CUDA graph, then a batched reduction writes
// their summaries; the persistent kernel runs the rest meanwhile. Their buffers use a 128-byte
// pitch for the fire kernel's 16-byte vector loads. The per-run data of both paths (start
// buffer, t0, steps, thresholds) is uploaded before each graph launch; the graph is captured
// again only when its shape changes (the large set, the number of passes, the geometry).
#include <algorithm>
#include <cstdarg>
#include <cstdio>
#include <cstring>
#include <numeric>
#include <string>
#include <vector>

#include "ensemble.cuh"
#include "fire_words.cuh"
#include "gbca_internal.cuh"
#include "measures.cuh"

namespace gbca {

namespace {

constexpr int kEnsThreads = 256;
constexpr int kEnsMaxHalo = 8;

// Bytes of each of a CTA's two shared buffers for tiles of TILE x TILE cells.
__host__ __device__ constexpr int ens_buf(int tile) { return (tile + 2 * kEnsMaxHalo) * (tile + 2 * kEnsMaxHalo); }

__device__ __forceinline__ bool fast_fire(const EnsInstance& I) {
    return I.rule == GBCA_RULE_FOREST_FIRE && I.nbhd == GBCA_VON_NEUMANN && I.radius == 1;
}

// The next state of the cell at offset o of a shared buffer with row pitch sx: the rule of
// src/rules.jl:385-389 / :446-456 or the forest fire, neighbours read from the buffer.
__device__ __forceinline__ int8_t ens_update(const EnsInstance& I, const int8_t* A, int sx, int o, uint64_t id,
                                             int64_t t, const DrawStep& ds, const PhiloxKeys& K, bool ff) {
    const int8_t c = A[o];
    if (ff) {
        if (c == 2) return 0;
        const bool empty = c == 0;
        if (!empty && (A[o - 1] == 2 || A[o + 1] == 2 || A[o - sx] == 2 || A[o + sx] == 2)) return 2;
        const bool hit = draw_below(draw_fast(ds, K, (uint32_t)id, empty ? 1u : 2u), empty ? I.thr_p : I.thr_f,
                                    I.params_f32 != 0);
        return empty ? (hit ? 1 : 0) : (hit ? 2 : 1);
    }
    const int r = I.radius;
    int n = 0;
    bool fire = false;
    for (int dj = -r; dj <= r; ++dj) {
        const int rr = I.nbhd == GBCA_MOORE ? r : r - (dj < 0 ? -dj : dj);
        const int8_t* row = A + o + dj * sx;
        for (int di = -rr; di <= rr; ++di) {
            if (di == 0 && dj == 0) continue;
            const int8_t v = row[di];
            n += v == 1;
            fire |= v == 2;
        }
    }
    if (I.rule == GBCA_RULE_LIFE) {
        const uint64_t mask = c == 1 ? I.survive : I.birth;
        return (int8_t)(n < 64 ? (mask >> n) & 1u : 0u);
    }
    if (I.rule == GBCA_RULE_GENERATIONS) {
        const int s = c;
        if (s == 0) return (int8_t)(n < 64 ? (I.birth >> n) & 1u : 0u);
        if (s == 1) {
            if (n < 64 && ((I.survive >> n) & 1u)) return c;
            return (int8_t)(I.states > 2 ? 2 : 0);
        }
        return (int8_t)(s + 1 < I.states ? s + 1 : 0);
    }
    if (c == 2) return 0;
    if (c == 0) return draw_below(cell_draw(I.seed, id, t, 1), I.thr_p, I.params_f32 != 0) ? 1 : 0;
    if (fire) return 2;
    return draw_below(cell_draw(I.seed, id, t, 2), I.thr_f, I.params_f32 != 0) ? 2 : 1;
}

__device__ __forceinline__ int8_t boundary_value(const EnsInstance& I, const int8_t* base, int64_t pitch, int64_t gx,
                                                 int64_t gy) {
    const int64_t mx = map_axis(I.bnd0, gx, I.n1), my = map_axis(I.bnd1, gy, I.n2);
    if (my < 0) return (int8_t)I.cval1;
    if (mx < 0) return (int8_t)I.cval0;
    return base[mx + my * pitch];
}

// The whole lattice in shared memory, padded by r on every side.
__device__ void run_in_smem(const EnsInstance& I, int8_t* pool, int8_t* A, int8_t* B, const PhiloxKeys& K) {
    const int r = I.radius, n1 = (int)I.n1, n2 = (int)I.n2, P1 = n1 + 2 * r;
    int8_t* g = pool + I.off[I.cur];
    for (int q = threadIdx.x; q < n1 * n2; q += blockDim.x) {
        const int x = q % n1, y = q / n1;
        A[(y + r) * P1 + x + r] = g[x + (int64_t)y * I.pitch];
    }
    const bool ff = fast_fire(I);
    const int ring = 2 * r * P1 + 2 * r * n2;  // halo cells
    for (int64_t s = 0; s < I.nsteps; ++s) {
        __syncthreads();
        for (int q = threadIdx.x; q < ring; q += blockDim.x) {  // refresh the halo from the interior
            int hx, hy;
            if (q < 2 * r * P1) {
                const int row = q / P1;
                hx = q % P1;
                hy = row < r ? row : n2 + row;  // rows 0..r-1 and n2+r..n2+2r-1
            } else {
                const int q2 = q - 2 * r * P1, col = q2 % (2 * r);
                hy = r + q2 / (2 * r);
                hx = col < r ? col : n1 + col;
            }
            A[hy * P1 + hx] = boundary_value(I, A + r * P1 + r, P1, hx - r, hy - r);
        }
        __syncthreads();
        const int64_t t = I.t0 + s;
        const DrawStep ds = draw_step(K, t);
        for (int q = threadIdx.x; q < n1 * n2; q += blockDim.x) {
            const int x = q % n1, y = q / n1, o = (y + r) * P1 + x + r;
            B[o] = ens_update(I, A, P1, o, (uint64_t)q + 1u, t, ds, K, ff);
        }
        int8_t* tmp = A; A = B; B = tmp;
    }
    __syncthreads();
    for (int q = threadIdx.x; q < n1 * n2; q += blockDim.x) {
        const int x = q % n1, y = q / n1;
        g[x + (int64_t)y * I.pitch] = A[(y + r) * P1 + x + r];
    }
}

// Tiles of TILE x TILE with I.depth-step temporal blocking through the two global
// buffers. Returns the buffer index holding the final state.
template <int TILE>
__device__ int run_tiled(const EnsInstance& I, int8_t* pool, int8_t* A0, int8_t* B0, const PhiloxKeys& K) {
    const int r = I.radius;
    const bool ff = fast_fire(I);
    const int Kmax = I.depth;  // steps per pass, depth * r <= kEnsMaxHalo
    const int ntx = (int)((I.n1 + TILE - 1) / TILE), nty = (int)((I.n2 + TILE - 1) / TILE);
    int cur = I.cur;
    for (int64_t s0 = 0; s0 < I.nsteps; s0 += Kmax) {
        const int k = (int)((I.nsteps - s0) < Kmax ? (I.nsteps - s0) : Kmax);
        const int H = k * r, S = TILE + 2 * H;
        const int8_t* src = pool + I.off[cur];
        int8_t* dst = pool + I.off[cur ^ 1];
        for (int tile = 0; tile < ntx * nty; ++tile) {
            const int64_t X0 = (int64_t)(tile % ntx) * TILE, Y0 = (int64_t)(tile / ntx) * TILE;
            int8_t* A = A0;
            int8_t* B = B0;
            __syncthreads();
            for (int q = threadIdx.x; q < S * S; q += blockDim.x) {
                const int lx = q % S, ly = q / S;
                A[q] = boundary_value(I, src, I.pitch, X0 - H + lx, Y0 - H + ly);
            }
            __syncthreads();
            for (int sub = 0; sub < k; ++sub) {
                const int64_t t = I.t0 + s0 + sub;
                const DrawStep ds = draw_step(K, t);
                const int ex = (k - 1 - sub) * r, lo = H - ex, w = TILE + 2 * ex;
                for (int q = threadIdx.x; q < w * w; q += blockDim.x) {
                    const int lx = lo + q % w, ly = lo + q / w, o = ly * S + lx;
                    const int64_t mx = map_axis(I.bnd0, X0 - H + lx, I.n1), my = map_axis(I.bnd1, Y0 - H + ly, I.n2);
                    if (mx < 0 || my < 0) {
                        B[o] = (int8_t)(my < 0 ? I.cval1 : I.cval0);
                        continue;
                    }
                    B[o] = ens_update(I, A, S, o, (uint64_t)(mx + my * I.n1) + 1u, t, ds, K, ff);
                }
                __syncthreads();
                int8_t* tmp = A; A = B; B = tmp;
            }
            for (int q = threadIdx.x; q < TILE * TILE; q += blockDim.x) {
                const int64_t gx = X0 + q % TILE, gy = Y0 + q / TILE;
                if (gx < I.n1 && gy < I.n2) dst[gx + gy * I.pitch] = A[(H + q / TILE) * S + H + q % TILE];
            }
        }
        __syncthreads();  // the whole pass is written before the next one reads it
        cur ^= 1;
    }
    return cur;
}

// Forest fire (VonNeumann(1)) with the whole lattice in shared memory, four cells per work
// item: cell (x, y) lives at byte (y + 1) * P1 + x + 4 of a row pitch P1 = 4 ceil((n1 + 8) / 4),
// so the interior starts on a word; the halo (row -1, row n2, column -1, column n1) is
// refreshed from the boundary map before every step.
__device__ void run_in_smem_fire(const EnsInstance& I, int8_t* pool, int8_t* A, int8_t* B, const PhiloxKeys& K,
                                 const FireGeom& g) {
    const int n1 = (int)I.n1, n2 = (int)I.n2, P1 = (n1 + 8 + 3) / 4 * 4;
    int8_t* gl = pool + I.off[I.cur];
    for (int q = threadIdx.x; q < n1 * n2; q += blockDim.x) {
        const int x = q % n1, y = q / n1;
        A[(y + 1) * P1 + x + 4] = gl[x + (int64_t)y * I.pitch];
    }
    const int ring = 2 * (n1 + 2) + 2 * n2;
    for (int64_t s = 0; s < I.nsteps; ++s) {
        __syncthreads();
        for (int q = threadIdx.x; q < ring; q += blockDim.x) {
            int x, y;
            if (q < 2 * (n1 + 2)) {
                x = q % (n1 + 2) - 1;
                y = q < n1 + 2 ? -1 : n2;
            } else {
                const int q2 = q - 2 * (n1 + 2);
                y = q2 >> 1;
                x = (q2 & 1) ? n1 : -1;
            }
            A[(y + 1) * P1 + x + 4] = boundary_value(I, A + P1 + 4, P1, x, y);
        }
        __syncthreads();
        const DrawStep ds = draw_step(K, I.t0 + s);
        fire_substep_words<false>((const uint32_t*)A, (uint32_t*)B, P1 / 4, 1, (n1 + 3) / 4, 1, n2, -4, -1, g, ds, K,
                                  threadIdx.x, blockDim.x, s == 0);
        int8_t* tmp = A; A = B; B = tmp;
    }
    __syncthreads();
    for (int q = threadIdx.x; q < n1 * n2; q += blockDim.x) {
        const int x = q % n1, y = q / n1;
        gl[x + (int64_t)y * I.pitch] = A[(y + 1) * P1 + x + 4];
    }
}

// Forest fire on tiles of TILE^2 through the two global buffers, I.depth (<= 8) steps per
// pass, four cells per work item. Returns the buffer holding the final state.
template <int TILE>
__device__ int run_tiled_fire(const EnsInstance& I, int8_t* pool, int8_t* A0, int8_t* B0, const PhiloxKeys& K,
                              const FireGeom& g) {
    constexpr int HX = kEnsMaxHalo, SX = TILE + 2 * HX, SW = SX / 4;
    const int ntx = (int)((I.n1 + TILE - 1) / TILE), nty = (int)((I.n2 + TILE - 1) / TILE);
    const int depth = I.depth;
    int cur = I.cur;
    for (int64_t s0 = 0; s0 < I.nsteps; s0 += depth) {
        const int k = (int)((I.nsteps - s0) < depth ? (I.nsteps - s0) : depth);
        const int SY = TILE + 2 * k;
        const int8_t* src = pool + I.off[cur];
        int8_t* dst = pool + I.off[cur ^ 1];
        for (int tile = 0; tile < ntx * nty; ++tile) {
            const int64_t X0 = (int64_t)(tile % ntx) * TILE, Y0 = (int64_t)(tile / ntx) * TILE;
            int8_t* A = A0;
            int8_t* B = B0;
            __syncthreads();
            for (int q = threadIdx.x; q < SX * SY; q += blockDim.x) {
                const int lx = q % SX, ly = q / SX;
                A[q] = boundary_value(I, src, I.pitch, X0 - HX + lx, Y0 - k + ly);
            }
            __syncthreads();
            const bool interior = X0 - HX >= 0 && X0 + TILE + HX <= I.n1 && Y0 - k >= 0 &&
                                  Y0 + TILE + k <= I.n2;
            for (int sub = 0; sub < k; ++sub) {
                const DrawStep ds = draw_step(K, I.t0 + s0 + sub);
                const int ex = k - 1 - sub;
                const int w_lo = (HX - ex) >> 2, w_hi = (HX + TILE + ex + 3) >> 2;
                const bool exact = s0 == 0 && sub == 0;  // the run's first step may read any Int8 value
                if (interior)
                    fire_substep_words<false>((const uint32_t*)A, (uint32_t*)B, SW, w_lo, w_hi - w_lo, k - ex,
                                              TILE + 2 * ex, X0 - HX, Y0 - k, g, ds, K, threadIdx.x, blockDim.x,
                                              exact);
                else
                    fire_substep_words<true>((const uint32_t*)A, (uint32_t*)B, SW, w_lo, w_hi - w_lo, k - ex,
                                             TILE + 2 * ex, X0 - HX, Y0 - k, g, ds, K, threadIdx.x, blockDim.x,
                                             exact);
                __syncthreads();
                int8_t* tmp = A; A = B; B = tmp;
            }
            for (int q = threadIdx.x; q < TILE * TILE; q += blockDim.x) {
                const int64_t gx = X0 + q % TILE, gy = Y0 + q / TILE;
                if (gx < I.n1 && gy < I.n2) dst[gx + gy * I.pitch] = A[(k + q / TILE) * SX + HX + q % TILE];
            }
        }
        __syncthreads();
        cur ^= 1;
    }
    return cur;
}

// Cell (i, j)'s share of the summary words: its value counted (0..7, else "other"), S, S2, and
// its VonNeumann(1) pairs' P, Q and W (a neighbour beyond a Constant edge is no neighbour).
__device__ __forceinline__ void summary_cell(const int8_t* base, int64_t pitch, int64_t n1, int64_t n2, int32_t bnd0,
                                             int32_t bnd1, int64_t i, int64_t j, long long* acc) {
    const int x = base[i + j * pitch];
    if (x >= 0 && x < kEnsCounts) {
#pragma unroll
        for (int v = 0; v < kEnsCounts; ++v) acc[v] += (x == v);
    } else {
        acc[kEnsCounts] += 1;
    }
    acc[kEnsCounts + 1] += x;
    acc[kEnsCounts + 2] += x * x;
    const int di[4] = {0, -1, 1, 0}, dj[4] = {-1, 0, 0, 1};
#pragma unroll
    for (int d = 0; d < 4; ++d) {
        const int64_t a = map_axis(bnd0, i + di[d], n1), b = map_axis(bnd1, j + dj[d], n2);
        if (a < 0 || b < 0) continue;
        const int y = base[a + b * pitch];
        acc[kEnsCounts + 3] += x * y;
        acc[kEnsCounts + 4] += x + y;
        acc[kEnsCounts + 5] += 1;
    }
}

// The block's summary words, reduced into red[] (zeroed by the caller before a barrier).
__device__ __forceinline__ void summary_reduce(const long long* acc, unsigned long long* red) {
#pragma unroll
    for (int k = 0; k < kEnsSumWords; ++k) {
        long long v = acc[k];
#pragma unroll
        for (int o = 16; o > 0; o >>= 1) v += __shfl_down_sync(0xffffffffu, v, o);
        if ((threadIdx.x & 31) == 0) atomicAdd(&red[k], (unsigned long long)v);
    }
    __syncthreads();
}

// Integer summaries of a state (values 0..7 counted, Moran's I sums over VonNeumann(1)).
__device__ __noinline__ void summarize(const EnsInstance& I, const int8_t* base, int64_t pitch, EnsSummary* out) {
    __shared__ unsigned long long red[kEnsSumWords];
    for (int k = threadIdx.x; k < kEnsSumWords; k += blockDim.x) red[k] = 0ull;
    __syncthreads();
    long long acc[kEnsSumWords];
#pragma unroll
    for (int k = 0; k < kEnsSumWords; ++k) acc[k] = 0;
    const int64_t n = I.n1 * I.n2;
    for (int64_t q = threadIdx.x; q < n; q += blockDim.x)
        summary_cell(base, pitch, I.n1, I.n2, I.bnd0, I.bnd1, q % I.n1, q / I.n1, acc);
    summary_reduce(acc, red);
    for (int k = threadIdx.x; k < kEnsSumWords; k += blockDim.x) out->w[k] = (long long)red[k];
}

// Summaries of the large instances after their batched passes: block b reduces output tile b
// of the jobs' concatenated tile order (launch_fire_batch's tiles) of the final buffer and adds
// its integers to the instance's summary words, zeroed earlier in the same graph. Integer sums
// in any order: the same words as summarize() on one CTA.
__global__ void __launch_bounds__(kEnsThreads) k_ens_measures(const FireJob* __restrict__ jobs,
                                                              const int32_t* __restrict__ tile_job, int K,
                                                              EnsSummary* __restrict__ out) {
    __shared__ unsigned long long red[kEnsSumWords];
    const FireJob& J = jobs[tile_job[blockIdx.x]];
    const int64_t passes = J.nsteps > 0 ? (J.nsteps + K - 1) / K : 0;
    const int8_t* base = J.buf[J.cur0 ^ (int)(passes & 1)];
    const int64_t n1 = J.p.n1, n2 = J.p.n2, pitch = J.p.pitch;
    const int local = (int)blockIdx.x - J.tile0;
    const int64_t X0 = (int64_t)(local % J.tiles_x) * kFireTileCols, Y0 = (int64_t)(local / J.tiles_x) * kFireTileRows;
    for (int k = threadIdx.x; k < kEnsSumWords; k += blockDim.x) red[k] = 0ull;
    __syncthreads();
    long long acc[kEnsSumWords];
#pragma unroll
    for (int k = 0; k < kEnsSumWords; ++k) acc[k] = 0;
    for (int q = threadIdx.x; q < kFireTileCols * kFireTileRows; q += blockDim.x) {
        const int64_t i = X0 + q % kFireTileCols, j = Y0 + q / kFireTileCols;
        if (i < n1 && j < n2) summary_cell(base, pitch, n1, n2, J.p.bnd[0], J.p.bnd[1], i, j, acc);
    }
    summary_reduce(acc, red);
    if (threadIdx.x < kEnsSumWords && red[threadIdx.x])
        atomicAdd((unsigned long long*)&out[J.inst].w[threadIdx.x], red[threadIdx.x]);
}

template <int TILE>
__global__ void __launch_bounds__(kEnsThreads) k_ensemble(const EnsInstance* __restrict__ insts,
                                                          const int* __restrict__ order, int n,
                                                          int* __restrict__ counter, int8_t* __restrict__ pool,
                                                          EnsSummary* __restrict__ out, int* __restrict__ final_cur) {
    extern __shared__ __align__(16) int8_t ens_smem[];
    int8_t* sA = ens_smem;
    int8_t* sB = ens_smem + ens_buf(TILE);
    __shared__ int s_q;
    for (;;) {
        __syncthreads();
        if (threadIdx.x == 0) s_q = atomicAdd(counter, 1);
        __syncthreads();
        const int q = s_q;
        if (q >= n) return;
        const int i = order[q];
        const EnsInstance I = insts[i];
        const PhiloxKeys K = philox_keys_dev(I.seed);
        int cur = I.cur;
        if (I.nsteps > 0) {
            if (fast_fire(I)) {
                FireGeom g;
                g.n1 = I.n1;
                g.n2 = I.n2;
                g.bnd0 = I.bnd0;
                g.bnd1 = I.bnd1;
                g.cst0 = (uint32_t)(uint8_t)I.cval0 * 0x01010101u;
                g.cst1 = (uint32_t)(uint8_t)I.cval1 * 0x01010101u;
                fire_thresholds(I.thr_p, I.thr_f, I.params_f32 != 0, g);
                g.exact_always = fire_odd_constant(I.bnd0, I.cval0, I.bnd1, I.cval1);
                g.col0 = 0;
                g.n2g = I.n2;
                if (I.small) run_in_smem_fire(I, pool, sA, sB, K, g);
                else cur = run_tiled_fire<TILE>(I, pool, sA, sB, K, g);
            } else if (I.small) {
                run_in_smem(I, pool, sA, sB, K);
            } else {
                cur = run_tiled<TILE>(I, pool, sA, sB, K);
            }
        }
        __syncthreads();
        if (I.summarize) summarize(I, pool + I.off[cur], I.pitch, &out[i]);
        if (threadIdx.x == 0) final_cur[i] = cur;
    }
}


int efail(int code, const char* fmt, ...) {
    char msg[512];
    va_list ap;
    va_start(ap, fmt);
    vsnprintf(msg, sizeof msg, fmt, ap);
    va_end(ap);
    set_last_error(msg);
    return code;
}

// The kernel for a tile size, with its shared memory opted in.
template <int TILE>
cudaError_t ens_kernel(void (**fn)(const EnsInstance*, const int*, int, int*, int8_t*, EnsSummary*, int*),
                       size_t* smem) {
    *fn = k_ensemble<TILE>;
    *smem = 2 * (size_t)ens_buf(TILE);
    return ensure_dynamic_smem((const void*)k_ensemble<TILE>, *smem);
}

cudaError_t ens_select(int tile, void (**fn)(const EnsInstance*, const int*, int, int*, int8_t*, EnsSummary*, int*),
                       size_t* smem) {
    switch (tile) {
        case 64: return ens_kernel<64>(fn, smem);
        case 192: return ens_kernel<192>(fn, smem);
        default: return ens_kernel<128>(fn, smem);
    }
}

}  // namespace

bool ensemble_tile_ok(int tile) { return tile == 64 || tile == 128 || tile == 192; }

cudaError_t launch_ensemble(const EnsInstance* d_inst, const int* d_order, int n, int* d_counter, int8_t* pool,
                            EnsSummary* d_out, int* d_cur, int grid, cudaStream_t st, int tile) {
    cudaError_t e = cudaMemsetAsync(d_counter, 0, sizeof(int), st);
    if (e != cudaSuccess) return e;
    void (*fn)(const EnsInstance*, const int*, int, int*, int8_t*, EnsSummary*, int*) = nullptr;
    size_t smem = 0;
    e = ens_select(tile, &fn, &smem);
    if (e != cudaSuccess) return e;
    fn<<<grid, kEnsThreads, smem, st>>>(d_inst, d_order, n, d_counter, pool, d_out, d_cur);
    count_launch();
    return cudaGetLastError();
}

int ensemble_grid(int tile) {
    int dev = 0, nsm = 0, per = 0;
    cudaGetDevice(&dev);
    cudaDeviceGetAttribute(&nsm, cudaDevAttrMultiProcessorCount, dev);
    void (*fn)(const EnsInstance*, const int*, int, int*, int8_t*, EnsSummary*, int*) = nullptr;
    size_t smem = 0;
    if (ens_select(tile, &fn, &smem) == cudaSuccess)
        cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per, fn, kEnsThreads, smem);
    cudaGetLastError();
    return nsm * (per > 0 ? per : 1);
}

int ensemble_smem_cells(int tile) { return ens_buf(tile); }

bool ensemble_fits_smem(const gbca_desc& d, int tile) {
    const int buf = ens_buf(tile);
    if (d.rule == GBCA_RULE_FOREST_FIRE && d.nbhd == GBCA_VON_NEUMANN && d.radius == 1)
        return (d.n1 + 8 + 3) / 4 * 4 * (d.n2 + 2) <= buf;
    return (d.n1 + 2 * d.radius) * (d.n2 + 2 * d.radius) <= buf;
}

bool ensemble_large_capable(const gbca_desc& d) {
    return d.rule == GBCA_RULE_FOREST_FIRE && d.nbhd == GBCA_VON_NEUMANN && d.radius == 1 &&
           d.scheme == GBCA_SYNCHRONOUS;
}

int ensemble_depth(const gbca_desc& d, int depth) {
    const int cap = kEnsMaxHalo / d.radius;  // the halo of a pass fits the tile's margin
    if (depth <= 0 || depth > cap) depth = cap;
    return depth < 1 ? 1 : depth;
}

}  // namespace gbca

using namespace gbca;

struct gbca_ensemble {
    int32_t n = 0;
    std::vector<gbca_desc> descs;
    std::vector<EnsInstance> h_inst;
    EnsInstance* d_inst = nullptr;
    int* d_order = nullptr;
    int* d_counter = nullptr;
    int* d_cur = nullptr;
    EnsSummary* d_out = nullptr;
    EnsSummary* h_out = nullptr;
    int* h_cur = nullptr;
    int8_t* pool = nullptr;
    size_t pool_bytes = 0;
    cudaStream_t stream = nullptr;
    cudaGraphExec_t exec = nullptr;
    int grid = 0;
    int tile = 128;   // the kernel's tile side (gbca_ensemble_set_geometry / gbca_ensemble_tune)
    int depth = 0;    // steps per pass of the tiled path; 0: the deepest the halo allows
    bool ran = false;
    // large instances: batched multi-lattice fire passes on a forked stream of the same graph
    int64_t large_cells = (int64_t)1 << 18;  // smallest large instance (cells); 0: none is large
    int large_k = 1;                          // steps per batched pass
    std::vector<int> big;                     // the large instances (create order)
    std::vector<int> big_final;               // their buffer after the last run
    std::vector<gbca::FireJob> h_jobs;
    gbca::FireJob* d_jobs = nullptr;
    int32_t* d_tile_job = nullptr;
    int cap_jobs = 0, cap_tiles = 0;
    int graph_kernels = 0;                    // kernel launches one replay of the graph makes
    cudaStream_t aux = nullptr;
    cudaEvent_t ev_fork = nullptr, ev_join = nullptr;
    std::vector<int64_t> graph_sig;           // the shape the captured graph runs
};

namespace {

// Applies a geometry: the small-lattice split and pass depth of every instance, the grid, and
// a fresh graph at the next run.
void apply_geometry(gbca_ensemble* e, int tile, int depth) {
    e->tile = tile;
    e->depth = depth;
    for (int32_t i = 0; i < e->n; ++i) {
        EnsInstance& I = e->h_inst[(size_t)i];
        I.small = ensemble_fits_smem(e->descs[(size_t)i], tile) ? 1 : 0;
        I.depth = ensemble_depth(e->descs[(size_t)i], depth);
    }
    e->grid = ensemble_grid(tile);
    if (e->exec) {
        cudaGraphExecDestroy(e->exec);
        e->exec = nullptr;
    }
}

// Whether instance i runs as batched multi-CTA passes under the current settings.
bool is_large(const gbca_ensemble* e, int32_t i) {
    const gbca_desc& d = e->descs[(size_t)i];
    const EnsInstance& I = e->h_inst[(size_t)i];
    return e->large_cells > 0 && ensemble_large_capable(d) && I.n1 * I.n2 >= e->large_cells &&
           I.n1 * I.n2 >= kEnsLargeFloor && I.pitch % 16 == 0;
}

// Captures one run: zero the work counter and the summaries; fork the batched passes of the
// large instances (one launch per pass, then their summaries) onto the second stream while the
// persistent kernel runs the others; join. Waits for the previous run first (its graph and job
// table are replaced).
cudaError_t capture_run(gbca_ensemble* e, const std::vector<int>& big, int ntiles, int n_small, int passes, int K) {
    cudaError_t c = cudaStreamSynchronize(e->stream);
    if (c != cudaSuccess) return c;
    if (e->exec) {
        cudaGraphExecDestroy(e->exec);
        e->exec = nullptr;
    }
    if (!big.empty()) {
        if (!e->aux) c = cudaStreamCreateWithFlags(&e->aux, cudaStreamNonBlocking);
        if (c == cudaSuccess && !e->ev_fork) c = cudaEventCreateWithFlags(&e->ev_fork, cudaEventDisableTiming);
        if (c == cudaSuccess && !e->ev_join) c = cudaEventCreateWithFlags(&e->ev_join, cudaEventDisableTiming);
        if (c == cudaSuccess && (size_t)e->cap_jobs < big.size()) {
            cudaFree(e->d_jobs);
            e->d_jobs = nullptr;
            c = cudaMalloc(&e->d_jobs, sizeof(FireJob) * big.size());
            e->cap_jobs = c == cudaSuccess ? (int)big.size() : 0;
        }
        if (c == cudaSuccess && e->cap_tiles < ntiles) {
            cudaFree(e->d_tile_job);
            e->d_tile_job = nullptr;
            c = cudaMalloc(&e->d_tile_job, sizeof(int32_t) * ntiles);
            e->cap_tiles = c == cudaSuccess ? ntiles : 0;
        }
        if (c == cudaSuccess) {  // block -> job map of the concatenated tile order
            std::vector<int32_t> tj((size_t)ntiles);
            for (size_t b = 0; b < big.size(); ++b) {
                const FireJob& J = e->h_jobs[b];
                const int end = b + 1 < big.size() ? e->h_jobs[b + 1].tile0 : ntiles;
                for (int t = J.tile0; t < end; ++t) tj[(size_t)t] = (int32_t)b;
            }
            c = cudaMemcpy(e->d_tile_job, tj.data(), sizeof(int32_t) * ntiles, cudaMemcpyHostToDevice);
        }
        if (c != cudaSuccess) return c;
    }
    void (*fn)(const EnsInstance*, const int*, int, int*, int8_t*, EnsSummary*, int*) = nullptr;
    size_t smem = 0;
    c = ens_select(e->tile, &fn, &smem);  // sets the kernel's shared-memory limit before capture
    if (c != cudaSuccess) return c;
    cudaGraph_t g = nullptr;
    c = cudaStreamBeginCapture(e->stream, cudaStreamCaptureModeRelaxed);
    if (c != cudaSuccess) return c;
    cudaError_t err = cudaMemsetAsync(e->d_counter, 0, sizeof(int), e->stream);
    if (err == cudaSuccess) err = cudaMemsetAsync(e->d_out, 0, sizeof(EnsSummary) * e->n, e->stream);
    if (err == cudaSuccess && !big.empty()) {
        err = cudaEventRecord(e->ev_fork, e->stream);
        if (err == cudaSuccess) err = cudaStreamWaitEvent(e->aux, e->ev_fork, 0);
    }
    int kernels = 0;
    if (err == cudaSuccess && n_small > 0) {
        fn<<<e->grid, kEnsThreads, smem, e->stream>>>(e->d_inst, e->d_order, n_small, e->d_counter, e->pool, e->d_out,
                                                      e->d_cur);
        err = cudaGetLastError();
        ++kernels;
    }
    if (err == cudaSuccess && !big.empty()) {
        for (int q = 0; q < passes && err == cudaSuccess; ++q, ++kernels)
            err = launch_fire_batch(e->d_jobs, e->d_tile_job, ntiles, q, K, e->aux);
        if (err == cudaSuccess) {
            k_ens_measures<<<ntiles, kEnsThreads, 0, e->aux>>>(e->d_jobs, e->d_tile_job, K, e->d_out);
            err = cudaGetLastError();
            ++kernels;
        }
        // the join is recorded even after an error, so the capture ends with one stream
        const cudaError_t j1 = cudaEventRecord(e->ev_join, e->aux);
        const cudaError_t j2 = cudaStreamWaitEvent(e->stream, e->ev_join, 0);
        if (err == cudaSuccess) err = j1 != cudaSuccess ? j1 : j2;
    }
    c = cudaStreamEndCapture(e->stream, &g);
    if (err == cudaSuccess) err = c;
    if (err == cudaSuccess) err = cudaGraphInstantiate(&e->exec, g, 0);
    if (g) cudaGraphDestroy(g);
    e->graph_kernels = kernels;
    return err;
}

}  // namespace

extern "C" {

int gbca_ensemble_create(const gbca_desc* descs, int32_t n, gbca_ensemble** out) {
    if (!out || !descs || n < 1) return efail(GBCA_ERR_ARGUMENT, "an ensemble needs at least one problem");
    *out = nullptr;
    std::vector<EnsInstance> inst((size_t)n);
    size_t off = 0;
    for (int32_t i = 0; i < n; ++i) {
        const gbca_desc& d = descs[i];
        int rc = gbca_check(&d);
        if (rc != GBCA_OK) return rc;
        if (d.rule == GBCA_RULE_LENIA) return efail(GBCA_ERR_UNSUPPORTED, "ensemble instance %d: Lenia is not batched", i);
        if (d.rule == GBCA_RULE_SI_FIELD)
            return efail(GBCA_ERR_UNSUPPORTED, "ensemble instance %d: kernel-field rules are not batched", i);
        if (d.scheme != GBCA_SYNCHRONOUS)
            return efail(GBCA_ERR_UNSUPPORTED, "ensemble instance %d: batched ensembles run Synchronous()", i);
        if (d.radius > kEnsMaxHalo)
            return efail(GBCA_ERR_UNSUPPORTED, "ensemble instance %d: radius %d above %d", i, d.radius, kEnsMaxHalo);
        if (d.n1 * d.n2 >= ((int64_t)1 << 32) - 1)
            return efail(GBCA_ERR_ARGUMENT, "ensemble instance %d: more than 2^32 - 2 cells", i);
        EnsInstance& I = inst[(size_t)i];
        std::memset(&I, 0, sizeof I);
        I.n1 = d.n1;
        I.n2 = d.n2;
        // instances that may run as batched multi-CTA passes get a 128-byte pitch
        I.pitch = ensemble_large_capable(d) && d.n1 * d.n2 >= kEnsLargeFloor ? (d.n1 + 127) / 128 * 128 : d.n1;
        I.off[0] = (int64_t)off;
        off += (size_t)(I.pitch * d.n2 + 255) / 256 * 256;
        I.off[1] = (int64_t)off;
        off += (size_t)(I.pitch * d.n2 + 255) / 256 * 256;
        I.rule = d.rule;
        I.nbhd = d.nbhd;
        I.radius = d.radius;
        I.states = d.states;
        I.birth = d.birth;
        I.survive = d.survive;
        I.seed = d.seed;
        I.params_f32 = d.params_f32;
        I.bnd0 = d.boundary[0];
        I.bnd1 = d.boundary[1];
        I.cval0 = d.boundary[0] == GBCA_CONSTANT ? (int32_t)d.constant[0] : 0;
        I.cval1 = d.boundary[1] == GBCA_CONSTANT ? (int32_t)d.constant[1] : 0;
        I.small = ensemble_fits_smem(d, 128) ? 1 : 0;
        I.depth = ensemble_depth(d, 0);
        I.summarize = 1;
    }
    if (gbca_device_count() < 1) return efail(GBCA_ERR_CUDA, "no CUDA device is visible");
    gbca_ensemble* e = new gbca_ensemble();
    e->n = n;
    e->descs.assign(descs, descs + n);
    e->h_inst = inst;
    e->pool_bytes = off;
    cudaError_t c = cudaStreamCreateWithFlags(&e->stream, cudaStreamNonBlocking);
    if (c == cudaSuccess) c = cudaMalloc(&e->pool, e->pool_bytes);
    if (c == cudaSuccess) c = cudaMalloc(&e->d_inst, sizeof(EnsInstance) * n);
    if (c == cudaSuccess) c = cudaMalloc(&e->d_order, sizeof(int) * n);
    if (c == cudaSuccess) c = cudaMalloc(&e->d_counter, sizeof(int));
    if (c == cudaSuccess) c = cudaMalloc(&e->d_cur, sizeof(int) * n);
    if (c == cudaSuccess) c = cudaMalloc(&e->d_out, sizeof(EnsSummary) * n);
    if (c == cudaSuccess) c = cudaMallocHost(&e->h_out, sizeof(EnsSummary) * n);
    if (c == cudaSuccess) c = cudaMallocHost(&e->h_cur, sizeof(int) * n);
    if (c == cudaSuccess) c = cudaMemsetAsync(e->pool, 0, e->pool_bytes, e->stream);
    if (c == cudaSuccess) c = cudaMemsetAsync(e->d_out, 0, sizeof(EnsSummary) * n, e->stream);
    if (c == cudaSuccess) c = cudaStreamSynchronize(e->stream);
    if (c != cudaSuccess) {
        const bool oom = c == cudaErrorMemoryAllocation;
        gbca_ensemble_destroy(e);
        cudaGetLastError();
        return oom ? efail(GBCA_ERR_OUT_OF_MEMORY, "ensemble allocation of %zu bytes failed", off)
                   : efail(GBCA_ERR_CUDA, "gbca_ensemble_create: %s", cudaGetErrorString(c));
    }
    e->grid = ensemble_grid(e->tile);
    *out = e;
    return GBCA_OK;
}

int gbca_ensemble_destroy(gbca_ensemble* e) {
    if (!e) return GBCA_OK;
    if (e->stream) cudaStreamSynchronize(e->stream);
    if (e->exec) cudaGraphExecDestroy(e->exec);
    cudaFree(e->pool);
    cudaFree(e->d_inst);
    cudaFree(e->d_order);
    cudaFree(e->d_counter);
    cudaFree(e->d_cur);
    cudaFree(e->d_out);
    if (e->h_out) cudaFreeHost(e->h_out);
    if (e->h_cur) cudaFreeHost(e->h_cur);
    cudaFree(e->d_jobs);
    cudaFree(e->d_tile_job);
    if (e->ev_fork) cudaEventDestroy(e->ev_fork);
    if (e->ev_join) cudaEventDestroy(e->ev_join);
    if (e->aux) cudaStreamDestroy(e->aux);
    if (e->stream) cudaStreamDestroy(e->stream);
    delete e;
    return GBCA_OK;
}

int gbca_ensemble_set_state(gbca_ensemble* e, int32_t i, const void* host, size_t nbytes) {
    if (!e || !host || i < 0 || i >= e->n) return efail(GBCA_ERR_ARGUMENT, "bad ensemble, instance or state");
    const EnsInstance& I = e->h_inst[(size_t)i];
    if (nbytes != (size_t)(I.n1 * I.n2))
        return efail(GBCA_ERR_STATE, "instance %d has %lld cells, the state %zu bytes", i, (long long)(I.n1 * I.n2),
                     nbytes);
    cudaError_t c = cudaMemcpy2DAsync(e->pool + I.off[I.cur], (size_t)I.pitch, host, (size_t)I.n1, (size_t)I.n1,
                                      (size_t)I.n2, cudaMemcpyHostToDevice, e->stream);
    if (c == cudaSuccess) c = cudaStreamSynchronize(e->stream);
    if (c != cudaSuccess) return efail(GBCA_ERR_CUDA, "ensemble set_state: %s", cudaGetErrorString(c));
    return GBCA_OK;
}

int gbca_ensemble_fill(gbca_ensemble* e, int32_t value) {
    if (!e) return efail(GBCA_ERR_ARGUMENT, "null ensemble");
    if (value < -128 || value > 127) return efail(GBCA_ERR_ARGUMENT, "fill value %d is not an Int8", value);
    cudaError_t c = cudaMemsetAsync(e->pool, value & 0xFF, e->pool_bytes, e->stream);
    if (c != cudaSuccess) return efail(GBCA_ERR_CUDA, "ensemble fill: %s", cudaGetErrorString(c));
    return GBCA_OK;
}

int gbca_ensemble_run(gbca_ensemble* e, const int64_t* t0, const int64_t* nsteps, const double* params,
                      int32_t nparams) {
    if (!e || !nsteps) return efail(GBCA_ERR_ARGUMENT, "null ensemble or step counts");
    std::vector<int64_t> work((size_t)e->n);
    for (int32_t i = 0; i < e->n; ++i) {
        EnsInstance& I = e->h_inst[(size_t)i];
        const gbca_desc& d = e->descs[(size_t)i];
        if (nsteps[i] < 0) return efail(GBCA_ERR_ARGUMENT, "instance %d: negative step count", i);
        I.t0 = t0 ? t0[i] : 0;
        I.nsteps = nsteps[i];
        if (d.rule == GBCA_RULE_FOREST_FIRE) {
            if (!params || nparams < 2) return efail(GBCA_ERR_ARGUMENT, "forest-fire instances need (p, f) each");
            I.thr_p = gbca_threshold(params[(size_t)i * nparams], d.params_f32);
            I.thr_f = gbca_threshold(params[(size_t)i * nparams + 1], d.params_f32);
        }
        work[(size_t)i] = I.n1 * I.n2 * (I.nsteps > 0 ? I.nsteps : 0);
    }
    // the large instances run as batched passes of K steps; the rest on the persistent kernel
    const int K = e->large_k;
    std::vector<int> big, order;
    int64_t passes = 0;
    for (int32_t i = 0; i < e->n; ++i) {
        if (is_large(e, i)) {
            big.push_back(i);
            const int64_t q = (e->h_inst[(size_t)i].nsteps + K - 1) / K;
            if (q > passes) passes = q;
        } else {
            order.push_back(i);
        }
    }
    std::stable_sort(order.begin(), order.end(), [&](int a, int b) { return work[(size_t)a] > work[(size_t)b]; });
    const int n_small = (int)order.size();
    // this run's jobs: the structure follows the large set, the rest the run's arguments
    e->h_jobs.resize(big.size());
    e->big_final.resize(big.size());
    int ntiles = 0;
    for (size_t b = 0; b < big.size(); ++b) {
        const int i = big[b];
        const EnsInstance& I = e->h_inst[(size_t)i];
        FireJob& J = e->h_jobs[b];
        std::memset(&J, 0, sizeof J);
        J.p = sweep_params(e->descs[(size_t)i], I.pitch, nullptr);
        J.p.thr_p = I.thr_p;
        J.p.thr_f = I.thr_f;
        J.p.keys = philox_keys(I.seed);
        J.p.t0 = I.t0;
        J.buf[0] = e->pool + I.off[0];
        J.buf[1] = e->pool + I.off[1];
        J.nsteps = I.nsteps;
        J.cur0 = I.cur;
        J.tiles_x = (int32_t)((I.n1 + kFireTileCols - 1) / kFireTileCols);
        J.tile0 = ntiles;
        J.inst = i;
        ntiles += J.tiles_x * (int32_t)((I.n2 + kFireTileRows - 1) / kFireTileRows);
        e->big_final[b] = I.cur ^ (int)(((I.nsteps + K - 1) / K) & 1);
    }
    std::vector<int64_t> sig = {e->tile, e->grid, K, n_small, passes, (int64_t)big.size()};
    sig.insert(sig.end(), big.begin(), big.end());
    cudaError_t c = cudaSuccess;
    if (!e->exec || sig != e->graph_sig) {
        c = capture_run(e, big, ntiles, n_small, (int)passes, K);
        if (c != cudaSuccess) {
            e->graph_sig.clear();
            cudaGetLastError();
            return efail(GBCA_ERR_CUDA, "ensemble graph capture: %s", cudaGetErrorString(c));
        }
        e->graph_sig = sig;
    }
    e->big = big;
    c = cudaMemcpyAsync(e->d_inst, e->h_inst.data(), sizeof(EnsInstance) * e->n, cudaMemcpyHostToDevice, e->stream);
    if (c == cudaSuccess && n_small > 0)
        c = cudaMemcpyAsync(e->d_order, order.data(), sizeof(int) * n_small, cudaMemcpyHostToDevice, e->stream);
    if (c == cudaSuccess && !big.empty())
        c = cudaMemcpyAsync(e->d_jobs, e->h_jobs.data(), sizeof(FireJob) * big.size(), cudaMemcpyHostToDevice,
                            e->stream);
    if (c != cudaSuccess) return efail(GBCA_ERR_CUDA, "ensemble upload: %s", cudaGetErrorString(c));
    c = cudaGraphLaunch(e->exec, e->stream);
    if (c != cudaSuccess) return efail(GBCA_ERR_CUDA, "ensemble launch: %s", cudaGetErrorString(c));
    count_launch(e->graph_kernels);
    // results come back with the summaries; the buffer holding each final state too
    c = cudaMemcpyAsync(e->h_cur, e->d_cur, sizeof(int) * e->n, cudaMemcpyDeviceToHost, e->stream);
    if (c != cudaSuccess) return efail(GBCA_ERR_CUDA, "ensemble result copy: %s", cudaGetErrorString(c));
    e->ran = true;
    return GBCA_OK;
}

int gbca_ensemble_sync(gbca_ensemble* e) {
    if (!e) return efail(GBCA_ERR_ARGUMENT, "null ensemble");
    cudaError_t c = cudaStreamSynchronize(e->stream);
    if (c != cudaSuccess) return efail(GBCA_ERR_CUDA, "ensemble sync: %s", cudaGetErrorString(c));
    if (e->ran) {
        std::vector<uint8_t> is_big((size_t)e->n, 0);
        for (size_t b = 0; b < e->big.size(); ++b) {
            e->h_inst[(size_t)e->big[b]].cur = e->big_final[b];
            is_big[(size_t)e->big[b]] = 1;
        }
        for (int32_t i = 0; i < e->n; ++i)
            if (!is_big[(size_t)i]) e->h_inst[(size_t)i].cur = e->h_cur[i];
        e->ran = false;
    }
    return GBCA_OK;
}

int gbca_ensemble_summaries(gbca_ensemble* e, int64_t* counts, int32_t nvals, int64_t* other, double* morans) {
    if (!e) return efail(GBCA_ERR_ARGUMENT, "null ensemble");
    if (nvals < 0 || nvals > kEnsCounts) return efail(GBCA_ERR_ARGUMENT, "nvals must be in 0:%d", kEnsCounts);
    int rc = gbca_ensemble_sync(e);
    if (rc != GBCA_OK) return rc;
    cudaError_t c = cudaMemcpyAsync(e->h_out, e->d_out, sizeof(EnsSummary) * e->n, cudaMemcpyDeviceToHost, e->stream);
    if (c == cudaSuccess) c = cudaStreamSynchronize(e->stream);
    if (c != cudaSuccess) return efail(GBCA_ERR_CUDA, "ensemble summaries: %s", cudaGetErrorString(c));
    for (int32_t i = 0; i < e->n; ++i) {
        const long long* w = e->h_out[i].w;
        const int64_t ncell = e->h_inst[(size_t)i].n1 * e->h_inst[(size_t)i].n2;
        int64_t inrange = 0;
        for (int v = 0; v < kEnsCounts; ++v) {
            if (v < nvals && counts) counts[(size_t)i * nvals + v] = w[v];
            if (v < nvals) inrange += w[v];
        }
        if (other) other[i] = ncell - inrange;
        if (morans)
            morans[i] = morans_from_sums(w[kEnsCounts + 1], w[kEnsCounts + 2], w[kEnsCounts + 3], w[kEnsCounts + 4],
                                         w[kEnsCounts + 5], ncell);
    }
    return GBCA_OK;
}

int gbca_ensemble_set_geometry(gbca_ensemble* e, int32_t tile, int32_t depth) {
    if (!e) return efail(GBCA_ERR_ARGUMENT, "null ensemble");
    if (!ensemble_tile_ok(tile)) return efail(GBCA_ERR_ARGUMENT, "ensemble tiles are 64, 128 or 192 cells, got %d", tile);
    if (depth < 0 || depth > kEnsMaxHalo)
        return efail(GBCA_ERR_ARGUMENT, "depth must lie in 0:%d (0: the deepest), got %d", kEnsMaxHalo, depth);
    int rc = gbca_ensemble_sync(e);
    if (rc != GBCA_OK) return rc;
    apply_geometry(e, tile, depth);
    return GBCA_OK;
}

int gbca_ensemble_set_large(gbca_ensemble* e, int64_t min_cells, int32_t steps_per_pass) {
    if (!e) return efail(GBCA_ERR_ARGUMENT, "null ensemble");
    if (min_cells != 0 && min_cells < kEnsLargeFloor)
        return efail(GBCA_ERR_ARGUMENT, "min_cells is 0 (none) or at least %lld, got %lld", (long long)kEnsLargeFloor,
                     (long long)min_cells);
    if (steps_per_pass < 1 || steps_per_pass > 16)
        return efail(GBCA_ERR_ARGUMENT, "steps_per_pass must lie in 1:16, got %d", steps_per_pass);
    int rc = gbca_ensemble_sync(e);
    if (rc != GBCA_OK) return rc;
    e->large_cells = min_cells;
    e->large_k = steps_per_pass;
    return GBCA_OK;
}

int gbca_ensemble_geometry(gbca_ensemble* e, int32_t* tile, int32_t* depth, int64_t* large_cells,
                           int32_t* large_steps, int32_t* n_large) {
    if (!e) return efail(GBCA_ERR_ARGUMENT, "null ensemble");
    if (tile) *tile = e->tile;
    if (depth) *depth = e->depth;
    if (large_cells) *large_cells = e->large_cells;
    if (large_steps) *large_steps = e->large_k;
    if (n_large) {
        int32_t k = 0;
        for (int32_t i = 0; i < e->n; ++i) k += is_large(e, i) ? 1 : 0;
        *n_large = k;
    }
    return GBCA_OK;
}

int gbca_ensemble_tune(gbca_ensemble* e, int64_t probe_steps, const double* params, int32_t nparams, int32_t* tile,
                       int32_t* depth) {
    if (!e) return efail(GBCA_ERR_ARGUMENT, "null ensemble");
    if (probe_steps < 1) return efail(GBCA_ERR_ARGUMENT, "probe_steps must be positive");
    int rc = gbca_ensemble_sync(e);
    if (rc != GBCA_OK) return rc;
    // keep the states and each instance's current buffer; every candidate starts from them
    std::vector<int32_t> cur0((size_t)e->n);
    for (int32_t i = 0; i < e->n; ++i) cur0[(size_t)i] = e->h_inst[(size_t)i].cur;
    int8_t* saved = nullptr;
    cudaEvent_t ev[2] = {nullptr, nullptr};
    cudaError_t c = cudaMalloc(&saved, e->pool_bytes);
    if (c == cudaSuccess) c = cudaMemcpyAsync(saved, e->pool, e->pool_bytes, cudaMemcpyDeviceToDevice, e->stream);
    if (c == cudaSuccess) c = cudaEventCreate(&ev[0]);
    if (c == cudaSuccess) c = cudaEventCreate(&ev[1]);
    const std::vector<int64_t> steps((size_t)e->n, probe_steps);
    struct Cand {
        int tile, depth;
        int64_t large_cells;
        int large_k;
    };
    // one candidate: restore the states, time the fastest of two probe runs
    auto probe = [&](const Cand& k, float* ms_min) {
        apply_geometry(e, k.tile, k.depth);
        e->large_cells = k.large_cells;
        e->large_k = k.large_k;
        *ms_min = -1.0f;
        for (int rep = 0; rep < 2 && c == cudaSuccess && rc == GBCA_OK; ++rep) {
            for (int32_t i = 0; i < e->n; ++i) e->h_inst[(size_t)i].cur = cur0[(size_t)i];
            c = cudaMemcpyAsync(e->pool, saved, e->pool_bytes, cudaMemcpyDeviceToDevice, e->stream);
            if (c == cudaSuccess) c = cudaEventRecord(ev[0], e->stream);
            if (c != cudaSuccess) break;
            rc = gbca_ensemble_run(e, nullptr, steps.data(), params, nparams);
            if (rc != GBCA_OK) break;
            c = cudaEventRecord(ev[1], e->stream);
            if (c == cudaSuccess) rc = gbca_ensemble_sync(e);
            float ms = 0.0f;
            if (c == cudaSuccess && rc == GBCA_OK) c = cudaEventElapsedTime(&ms, ev[0], ev[1]);
            if (*ms_min < 0.0f || ms < *ms_min) *ms_min = ms;
        }
        return c == cudaSuccess && rc == GBCA_OK;
    };
    // first the persistent kernel's tile and depth (large instances at the current split), then
    // the split: which instances run as batched passes, and the passes' depth
    const int tiles[3] = {64, 128, 192}, depths[3] = {2, 4, 0};
    float best = -1.0f;
    Cand win = {e->tile, e->depth, e->large_cells, e->large_k};
    const int64_t cells0 = e->large_cells;
    const int k0 = e->large_k;
    for (int a = 0; a < 3; ++a)
        for (int b = 0; b < 3; ++b) {
            const Cand k = {tiles[a], depths[b], cells0, k0};
            float ms = 0.0f;
            if (!probe(k, &ms)) break;
            if (best < 0.0f || ms < best) {
                best = ms;
                win = k;
            }
        }
    bool capable = false;
    for (int32_t i = 0; i < e->n; ++i)
        capable = capable || (ensemble_large_capable(e->descs[(size_t)i]) &&
                              e->h_inst[(size_t)i].n1 * e->h_inst[(size_t)i].n2 >= kEnsLargeFloor);
    if (capable && c == cudaSuccess && rc == GBCA_OK) {
        const int64_t splits[7] = {kEnsLargeFloor,     (int64_t)1 << 15, (int64_t)1 << 16, (int64_t)1 << 17,
                                   (int64_t)1 << 18, (int64_t)1 << 20, 0};
        const int ks[3] = {1, 2, 4};
        for (int a = 0; a < 7; ++a)
            for (int b = 0; b < 3; ++b) {
                if (splits[a] == 0 && b > 0) break;  // nothing runs as batched passes
                const Cand k = {win.tile, win.depth, splits[a], ks[b]};
                float ms = 0.0f;
                if (!probe(k, &ms)) break;
                if (ms < best) {
                    best = ms;
                    win = k;
                }
            }
    }
    e->large_cells = win.large_cells;
    e->large_k = win.large_k;
    const int best_tile = win.tile, best_depth = win.depth;
    for (int32_t i = 0; i < e->n; ++i) e->h_inst[(size_t)i].cur = cur0[(size_t)i];
    if (saved) {
        const cudaError_t c2 = cudaMemcpyAsync(e->pool, saved, e->pool_bytes, cudaMemcpyDeviceToDevice, e->stream);
        const cudaError_t c3 = cudaStreamSynchronize(e->stream);
        if (c == cudaSuccess) c = c2 != cudaSuccess ? c2 : c3;
        cudaFree(saved);
    }
    for (cudaEvent_t x : ev)
        if (x) cudaEventDestroy(x);
    apply_geometry(e, best_tile, best_depth);
    if (rc != GBCA_OK) return rc;
    if (c != cudaSuccess) {
        cudaGetLastError();
        return c == cudaErrorMemoryAllocation
                   ? efail(GBCA_ERR_OUT_OF_MEMORY, "the tuner's copy of the ensemble (%zu bytes) did not fit",
                           e->pool_bytes)
                   : efail(GBCA_ERR_CUDA, "ensemble tuning: %s", cudaGetErrorString(c));
    }
    if (tile) *tile = best_tile;
    if (depth) *depth = best_depth;
    return GBCA_OK;
}

int gbca_ensemble_get_state(gbca_ensemble* e, int32_t i, void* host, size_t nbytes) {
    if (!e || !host || i < 0 || i >= e->n) return efail(GBCA_ERR_ARGUMENT, "bad ensemble, instance or buffer");
    int rc = gbca_ensemble_sync(e);
    if (rc != GBCA_OK) return rc;
    const EnsInstance& I = e->h_inst[(size_t)i];
    if (nbytes != (size_t)(I.n1 * I.n2))
        return efail(GBCA_ERR_STATE, "instance %d has %lld cells, the buffer %zu bytes", i, (long long)(I.n1 * I.n2),
                     nbytes);
    cudaError_t c = cudaMemcpy2DAsync(host, (size_t)I.n1, e->pool + I.off[I.cur], (size_t)I.pitch, (size_t)I.n1,
                                      (size_t)I.n2, cudaMemcpyDeviceToHost, e->stream);
    if (c == cudaSuccess) c = cudaStreamSynchronize(e->stream);
    if (c != cudaSuccess) return efail(GBCA_ERR_CUDA, "ensemble get_state: %s", cudaGetErrorString(c));
    return GBCA_OK;
}

}  // extern "C"
