// sweep_life.cu — placeholder until the box-sum Life-like kernel lands.
#include "gbca_internal.cuh"

namespace gbca {
bool life_simd_supported(const SweepParams&) { return false; }
cudaError_t launch_life_simd(const SweepParams&, const int8_t*, int8_t*, cudaStream_t) { return cudaErrorNotSupported; }
}  // namespace gbca
