// sweep_life_vn6.cu — the bit-sliced sweep's kernels for von Neumann(6) (life_kernel.cuh): Life-like
// rules, the count kept running down each column.
#include "life_kernel.cuh"

namespace gbca {
template cudaError_t launch_life_vn<6>(const SweepParams&, const LifeGeom&, const LifeTables&, const int8_t*, int8_t*,
                                       cudaStream_t, int);
}  // namespace gbca
