// life_common.cuh — what the bit-sliced Life / Generations sweep shares between its host
// side (sweep_life.cu: rule tables, geometry, dispatch) and the per-radius translation units
// that instantiate its kernels (sweep_life_r*.cu, split so that they compile in parallel).
#pragma once

#include "gbca_internal.cuh"

namespace gbca {

constexpr int kMaxIntervals = 8;
constexpr int kLifeThreads = 256;

struct LifeTables {
    int32_t n[2];                                // interval counts: [0] dead cells, [1] live cells
    uint32_t m[2][kMaxIntervals][2][8];          // [kind][interval][lo, hi+1][bit] majority masks
    uint32_t c3, c4;                             // Generations: ~0 when C > 2, when C == 4
    uint32_t cb[3];                              // Generations, three planes: C's bits as masks
};

struct LifeGeom {
    int32_t tw, hw;   // core words, halo words (each side) per row
    int32_t ty, hy;   // core rows, halo rows (each side)
    int32_t sw, sy;   // smem row pitch in words (tw + 2hw + 2 guards), rows (ty + 2hy)
    int32_t K;        // sub-steps
};

// A sub-step's gate (mode 0: every cell updates, 1: Checkerboard parity `gate`, 2: the
size_t life_smem_bytes(const SweepParams& p, const LifeGeom& g);
// Bit planes per cell: 1 for Life, 2 for Generations with C <= 4, 3 up to C = 8.
inline int life_planes(const SweepParams& p) {
    return p.rule != GBCA_RULE_GENERATIONS ? 1 : (p.states <= 4 ? 2 : 3);
}

// The bit-sliced kernel for Moore(R) (Life-like, and Generations for R <= 2), one per
// translation unit sweep_life_rR.cu; ntiles > 0 runs the listed tiles of p.tile_list.
template <int R>
cudaError_t launch_life_radius(const SweepParams& p, const LifeGeom& g, const LifeTables& tb, const int8_t* src,
                               int8_t* dst, cudaStream_t st, int ntiles);
// The same for von Neumann(R), R = 1..7 (sweep_life_vnR.cu; Generations for R <= 3).
template <int R>
cudaError_t launch_life_vn(const SweepParams& p, const LifeGeom& g, const LifeTables& tb, const int8_t* src,
                           int8_t* dst, cudaStream_t st, int ntiles);

}  // namespace gbca
