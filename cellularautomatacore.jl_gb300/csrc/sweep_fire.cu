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
#include "fire_words.cuh"
#include "gbca_internal.cuh"

namespace gbca {

namespace {

constexpr int kFireTX = 256, kFireTY = 128;
constexpr int kFireThreadsX = 32, kFireThreadsY = 16;

// Four cells (one 32-bit word of the shared tile) per work item: neighbour tests in byte
// SIMD, then four independent Philox chains.
template <bool INTERIOR>
__device__ __forceinline__ void fire_tile(const SweepParams& p, const int8_t* __restrict__ src,
                                          int8_t* __restrict__ dst, int8_t* A, int8_t* B) {
    const int hx = p.halo_x, hy = p.halo_y;
    const int sx = kFireTX + 2 * hx, sy = kFireTY + 2 * hy;
    const int sw = sx / 4;  // words per shared row
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

    FireGeom g;
    g.n1 = p.n1;
    g.n2 = p.n2;
    g.bnd0 = p.bnd[0];
    g.bnd1 = p.bnd[1];
    g.cst0 = (uint32_t)(uint8_t)p.cval[0] * 0x01010101u;
    g.cst1 = (uint32_t)(uint8_t)p.cval[1] * 0x01010101u;
    fire_thresholds(p.thr_p, p.thr_f, p.params_f32 != 0, g);
    g.exact_always = fire_odd_constant(p.bnd[0], p.cval[0], p.bnd[1], p.cval[1]);
    for (int s = 0; s < p.nsub; ++s) {
        const DrawStep ds = draw_step(p.keys, p.t0 + s);
        const int ex = p.nsub - 1 - s;
        const int w_lo = (hx - ex) >> 2, w_hi = (hx + kFireTX + ex + 3) >> 2;  // words covering the region
        fire_substep_words<!INTERIOR>((const uint32_t*)A, (uint32_t*)B, sw, w_lo, w_hi - w_lo, hy - ex,
                                      kFireTY + 2 * ex, X0 - hx, Y0 - hy, g, ds, p.keys, tid, nthr,
                                      s == 0 && !p.states_valid);
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
    return !p.mask && p.rule == GBCA_RULE_FOREST_FIRE && p.nbhd == GBCA_VON_NEUMANN && p.radius == 1 &&
           p.scheme == GBCA_SYNCHRONOUS && p.n1 * p.n2 < ((int64_t)1 << 32) - 1 && p.pitch % 16 == 0;
}

cudaError_t launch_fire(const SweepParams& p0, const int8_t* src, int8_t* dst, cudaStream_t st) {
    SweepParams p = p0;
    p.tile_x = kFireTX;
    p.tile_y = kFireTY;
    p.halo_y = p.nsub;
    p.halo_x = (p.nsub + 15) / 16 * 16;
    p.keys = philox_keys(p.seed);
    const size_t smem = 2 * (size_t)(kFireTX + 2 * p.halo_x) * (size_t)(kFireTY + 2 * p.halo_y);
    cudaError_t e = cudaFuncSetAttribute(k_fire, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
    if (e != cudaSuccess) return e;
    dim3 grid((unsigned)((p.n1 + kFireTX - 1) / kFireTX), (unsigned)((p.n2 + kFireTY - 1) / kFireTY));
    k_fire<<<grid, dim3(kFireThreadsX, kFireThreadsY), smem, st>>>(p, src, dst);
    return cudaGetLastError();
}

}  // namespace gbca
