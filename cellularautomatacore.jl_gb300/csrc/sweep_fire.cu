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
#include "gbca_internal.cuh"

namespace gbca {

namespace {

constexpr int kFireTX = 256, kFireTY = 128;
constexpr int kFireThreadsX = 32, kFireThreadsY = 16;

// One draw site for both draw indices, so that lanes of a warp holding empty cells
// (draw 1) and trees (draw 2) share one Philox evaluation instead of running two.
__device__ __forceinline__ int8_t fire_cell(int8_t c, const int8_t* a, int sx, const DrawStep& ds, uint32_t id,
                                            uint64_t thr_p, uint64_t thr_f, bool f32) {
    if (c == 2) return 0;
    const bool empty = c == 0;
    if (!empty && (a[-1] == 2 || a[1] == 2 || a[-sx] == 2 || a[sx] == 2)) return 2;
    const bool hit = draw_below(draw_fast(ds, id, empty ? 1u : 2u), empty ? thr_p : thr_f, f32);
    return empty ? (hit ? 1 : 0) : (hit ? 2 : 1);
}

template <bool INTERIOR>
__device__ __forceinline__ void fire_tile(const SweepParams& p, const int8_t* __restrict__ src,
                                          int8_t* __restrict__ dst, int8_t* A, int8_t* B) {
    const int hx = p.halo_x, hy = p.halo_y;
    const int sx = kFireTX + 2 * hx, sy = kFireTY + 2 * hy;
    const int64_t X0 = (int64_t)blockIdx.x * kFireTX, Y0 = (int64_t)blockIdx.y * kFireTY;
    const int tid = threadIdx.y * kFireThreadsX + threadIdx.x;
    const int nthr = kFireThreadsX * kFireThreadsY;

    if (INTERIOR) {  // 16-byte loads: X0 - hx, sx and the pitch are multiples of 16
        const int qx = sx / 16;
        for (int q = tid; q < qx * sy; q += nthr) {
            const int lq = q % qx, ly = q / qx;
            const int4 v = *(const int4*)(src + (X0 - hx + 16 * lq) + (Y0 - hy + ly) * p.pitch);
            *(int4*)(A + ly * sx + 16 * lq) = v;
        }
    } else {
        for (int idx = tid; idx < sx * sy; idx += nthr) {
            const int lx = idx % sx, ly = idx / sx;
            const int64_t mx = map_axis(p.bnd[0], X0 - hx + lx, p.n1), my = map_axis(p.bnd[1], Y0 - hy + ly, p.n2);
            A[idx] = my < 0 ? (int8_t)p.cval[1] : (mx < 0 ? (int8_t)p.cval[0] : src[mx + my * p.pitch]);
        }
    }
    __syncthreads();

    const bool f32 = p.params_f32 != 0;
    for (int s = 0; s < p.nsub; ++s) {
        const DrawStep ds = draw_step(p.seed, p.t0 + s);
        const int ex = p.nsub - 1 - s;
        const int x_lo = hx - ex, x_hi = hx + kFireTX + ex;
        const int y_lo = hy - ex, y_hi = hy + kFireTY + ex;
        for (int ly = y_lo + threadIdx.y; ly < y_hi; ly += kFireThreadsY) {
            const int64_t gy = Y0 - hy + ly;
            int64_t my = gy;
            if (!INTERIOR) my = map_axis(p.bnd[1], gy, p.n2);
            for (int lx = x_lo + threadIdx.x; lx < x_hi; lx += kFireThreadsX) {
                int64_t mx = X0 - hx + lx;
                const int o = ly * sx + lx;
                if (!INTERIOR) {
                    mx = map_axis(p.bnd[0], mx, p.n1);
                    if (mx < 0 || my < 0) {
                        B[o] = (int8_t)(my < 0 ? p.cval[1] : p.cval[0]);
                        continue;
                    }
                }
                const uint32_t id = (uint32_t)(mx + my * p.n1 + 1);
                B[o] = fire_cell(A[o], A + o, sx, ds, id, p.thr_p, p.thr_f, f32);
            }
        }
        __syncthreads();
        int8_t* t = A; A = B; B = t;
    }

    if (INTERIOR) {
        const int qx = kFireTX / 16;
        for (int q = tid; q < qx * kFireTY; q += nthr) {
            const int lq = q % qx, oy = q / qx;
            *(int4*)(dst + (X0 + 16 * lq) + (Y0 + oy) * p.pitch) = *(const int4*)(A + (hy + oy) * sx + hx + 16 * lq);
        }
    } else {
        for (int idx = tid; idx < kFireTX * kFireTY; idx += nthr) {
            const int ox = idx % kFireTX, oy = idx / kFireTX;
            const int64_t gx = X0 + ox, gy = Y0 + oy;
            if (gx < p.n1 && gy < p.n2) dst[gx + gy * p.pitch] = A[(hy + oy) * sx + hx + ox];
        }
    }
}

__global__ void __launch_bounds__(kFireThreadsX* kFireThreadsY) k_fire(SweepParams p, const int8_t* __restrict__ src,
                                                                      int8_t* __restrict__ dst) {
    extern __shared__ __align__(16) int8_t smem_f[];
    const int sx = kFireTX + 2 * p.halo_x, sy = kFireTY + 2 * p.halo_y;
    int8_t* A = smem_f;
    int8_t* B = smem_f + sx * sy;
    const int64_t X0 = (int64_t)blockIdx.x * kFireTX, Y0 = (int64_t)blockIdx.y * kFireTY;
    const bool interior = X0 - p.halo_x >= 0 && X0 + kFireTX + p.halo_x <= p.n1 && Y0 - p.halo_y >= 0 &&
                          Y0 + kFireTY + p.halo_y <= p.n2;
    if (interior) fire_tile<true>(p, src, dst, A, B);
    else fire_tile<false>(p, src, dst, A, B);
}

}  // namespace

bool fire_fast_supported(const SweepParams& p) {
    return p.rule == GBCA_RULE_FOREST_FIRE && p.nbhd == GBCA_VON_NEUMANN && p.radius == 1 &&
           p.scheme == GBCA_SYNCHRONOUS && p.n1 * p.n2 < ((int64_t)1 << 32) - 1 && p.pitch % 16 == 0;
}

cudaError_t launch_fire(const SweepParams& p0, const int8_t* src, int8_t* dst, cudaStream_t st) {
    SweepParams p = p0;
    p.tile_x = kFireTX;
    p.tile_y = kFireTY;
    p.halo_y = p.nsub;
    p.halo_x = (p.nsub + 15) / 16 * 16;
    const size_t smem = 2 * (size_t)(kFireTX + 2 * p.halo_x) * (size_t)(kFireTY + 2 * p.halo_y);
    cudaError_t e = cudaFuncSetAttribute(k_fire, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
    if (e != cudaSuccess) return e;
    dim3 grid((unsigned)((p.n1 + kFireTX - 1) / kFireTX), (unsigned)((p.n2 + kFireTY - 1) / kFireTY));
    k_fire<<<grid, dim3(kFireThreadsX, kFireThreadsY), smem, st>>>(p, src, dst);
    return cudaGetLastError();
}

}  // namespace gbca
