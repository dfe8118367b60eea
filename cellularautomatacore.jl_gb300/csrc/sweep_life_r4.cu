// sweep_life_r4.cu — the bit-sliced sweep's kernels for Moore(4) (life_kernel.cuh).
#include "life_kernel.cuh"

namespace gbca {
template cudaError_t launch_life_radius<4>(const SweepParams&, const LifeGeom&, const LifeTables&, const int8_t*,
                                             int8_t*, cudaStream_t, int);
}  // namespace gbca
