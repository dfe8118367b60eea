// sweep_life_vn1.cu — the bit-sliced sweep's kernels for von Neumann(1) (life_kernel.cuh): Life-like
// rules and Generations with up to 8 states.
#include "life_kernel.cuh"

namespace gbca {
template cudaError_t launch_life_vn<1>(const SweepParams&, const LifeGeom&, const LifeTables&, const int8_t*, int8_t*,
                                       cudaStream_t, int);
}  // namespace gbca
