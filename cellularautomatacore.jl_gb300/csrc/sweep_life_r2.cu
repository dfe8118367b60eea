// sweep_life_r2.cu — the bit-sliced sweep's kernels for Moore(2) (life_kernel.cuh).
#include "life_kernel.cuh"

namespace gbca {
template cudaError_t launch_life_radius<2>(const SweepParams&, const LifeGeom&, const LifeTables&, const int8_t*,
                                             int8_t*, cudaStream_t, int);
}  // namespace gbca
