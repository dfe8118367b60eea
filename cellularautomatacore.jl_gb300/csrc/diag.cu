// diag.cu — the measured compute roof of the stochastic sweeps: how many Philox4x32-10 cell
// draws (the draw of src/random.jl:102-107 followed by its bernoulli compare, random.jl:129)
// this GPU completes per second when it does nothing else. The forest-fire kernel makes one
// such draw per cell-update, so this rate bounds it whatever the memory system does.
#include "gbca_internal.cuh"

namespace gbca {

namespace {

__global__ void __launch_bounds__(256) k_philox_roof(PhiloxKeys K, int64_t t, uint32_t per_thread, uint64_t thr,
                                                     uint32_t* __restrict__ out) {
    const DrawStep ds = draw_step(K, t);
    const uint32_t tid = blockIdx.x * blockDim.x + threadIdx.x;
    const uint32_t stride = gridDim.x * blockDim.x;
    uint32_t id = tid + 1u, hits = 0;
    for (uint32_t i = 0; i < per_thread; ++i, id += stride) {
        const uint2 w = draw_fast(ds, K, id, 1u + (i & 1u));
        hits += ((((uint64_t)w.x) << 32) | (uint64_t)w.y) < thr ? 1u : 0u;
    }
    out[tid] = hits;  // keeps every draw live
}

}  // namespace

}  // namespace gbca

extern "C" int gbca_philox_rate(int64_t draws, double* draws_per_s) {
    using namespace gbca;
    if (!draws_per_s || draws < 1) {
        set_last_error("gbca_philox_rate needs a positive draw count and an output");
        return GBCA_ERR_ARGUMENT;
    }
    *draws_per_s = 0.0;
    int dev = 0, nsm = 0;
    cudaGetDevice(&dev);
    cudaDeviceGetAttribute(&nsm, cudaDevAttrMultiProcessorCount, dev);
    const uint32_t threads = 256, blocks = (uint32_t)nsm * 8u;  // 2048 threads per SM
    const uint64_t total_threads = (uint64_t)threads * blocks;
    uint64_t per = ((uint64_t)draws + total_threads - 1) / total_threads;
    if (per > 0xFFFFFFFFull) per = 0xFFFFFFFFull;
    uint32_t* out = nullptr;
    cudaEvent_t e0 = nullptr, e1 = nullptr;
    cudaError_t e = cudaMalloc(&out, total_threads * sizeof(uint32_t));
    if (e == cudaSuccess) e = cudaEventCreate(&e0);
    if (e == cudaSuccess) e = cudaEventCreate(&e1);
    const PhiloxKeys K = philox_keys(3);
    const uint64_t thr = gbca_threshold(0.03, 0) << 11;
    float ms = 0.0f;
    if (e == cudaSuccess) {
        k_philox_roof<<<blocks, threads>>>(K, 0, (uint32_t)(per / 8 + 1), thr, out);  // warm-up
        count_launch();
        e = cudaEventRecord(e0);
    }
    if (e == cudaSuccess) {
        k_philox_roof<<<blocks, threads>>>(K, 1, (uint32_t)per, thr, out);
        count_launch();
        e = cudaGetLastError();
    }
    if (e == cudaSuccess) e = cudaEventRecord(e1);
    if (e == cudaSuccess) e = cudaEventSynchronize(e1);
    if (e == cudaSuccess) e = cudaEventElapsedTime(&ms, e0, e1);
    if (e0) cudaEventDestroy(e0);
    if (e1) cudaEventDestroy(e1);
    cudaFree(out);
    if (e != cudaSuccess) {
        set_last_error(cudaGetErrorString(e));
        return GBCA_ERR_CUDA;
    }
    *draws_per_s = (double)(per * total_threads) / (ms * 1e-3);
    return GBCA_OK;
}
