// sweep_life_vn1.cu — the bit-sliced sweep's kernels for von Neumann(1) (life_kernel.cuh): Life-like
// rules and Generations with up to 4 states.
#include "life_kernel.cuh"

namespace gbca {
cudaError_t launch_life_vn1(const SweepParams& p, const LifeGeom& g, const LifeTables& tb, const int8_t* src,
                            int8_t* dst, cudaStream_t st, int ntiles) {
    if (p.rule == GBCA_RULE_GENERATIONS) return launch_r<1, 2, true>(p, g, tb, src, dst, st, ntiles);
    return launch_r<1, 1, true>(p, g, tb, src, dst, st, ntiles);
}
}  // namespace gbca
