// sweep_life_r6.cu — the bit-sliced sweep's kernels for Moore(6) (life_kernel.cuh).
#include "life_kernel.cuh"

namespace gbca {
template cudaError_t launch_life_radius<6>(const SweepParams&, const LifeGeom&, const LifeTables&, const int8_t*,
                                             int8_t*, cudaStream_t, int);
}  // namespace gbca
