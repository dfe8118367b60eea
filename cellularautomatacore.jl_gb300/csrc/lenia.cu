// lenia.cu — placeholder until the Float32 Lenia kernels land.
#include "lenia.cuh"

namespace gbca {

struct LeniaPlan {
    int dummy;
};

int lenia_create(const gbca_desc&, int64_t, cudaStream_t, LeniaPlan** out, std::string& err) {
    *out = nullptr;
    err = "Lenia is not built yet";
    return GBCA_ERR_UNSUPPORTED;
}
void lenia_destroy(LeniaPlan* plan) { delete plan; }
int lenia_advance(LeniaPlan*, const float*, float*, int64_t, cudaStream_t, int*, void* const*, std::string& err) {
    err = "Lenia is not built yet";
    return GBCA_ERR_UNSUPPORTED;
}

}  // namespace gbca
