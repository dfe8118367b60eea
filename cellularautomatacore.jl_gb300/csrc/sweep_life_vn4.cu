// sweep_life_vn4.cu — the bit-sliced sweep's kernels for von Neumann(4) (life_kernel.cuh): Life-like
// rules, the count kept running down each column.
#include "life_kernel.cuh"

namespace gbca {
template cudaError_t launch_life_vn<4>(const SweepParams&, const LifeGeom&, const LifeTables&, const int8_t*, int8_t*,
                                       cudaStream_t, int);
}  // namespace gbca
