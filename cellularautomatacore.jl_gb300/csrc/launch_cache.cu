// launch_cache.cu — per-device facts the launchers need on every launch, looked up once.
//
// A launch of a small lattice's sweep takes a few microseconds on the GPU, so host calls that
// cost as much (setting a kernel's shared-memory limit, occupancy queries) would bound it; the
// launchers ask here instead, and the runtime is called only the first time.
#include <map>
#include <mutex>
#include <tuple>

#include "gbca_internal.cuh"

namespace gbca {

namespace {

std::mutex g_mu;
std::map<std::pair<const void*, int>, size_t> g_smem;                      // limit set per kernel, device
std::map<int, int> g_sms;                                                  // SMs per device
std::map<int, int> g_optin;                                                // opt-in shared memory per block
std::map<std::tuple<const void*, int, int, size_t>, int> g_blocks;         // resident blocks per SM

int current_device() {
    int dev = 0;
    cudaGetDevice(&dev);
    return dev;
}

}  // namespace

cudaError_t ensure_dynamic_smem(const void* fn, size_t bytes) {
    const int dev = current_device();
    std::lock_guard<std::mutex> lock(g_mu);
    size_t& cur = g_smem[{fn, dev}];
    if (bytes <= cur) return cudaSuccess;
    const cudaError_t e = cudaFuncSetAttribute(fn, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)bytes);
    if (e == cudaSuccess) cur = bytes;
    return e;
}

int device_sms() {
    const int dev = current_device();
    std::lock_guard<std::mutex> lock(g_mu);
    auto it = g_sms.find(dev);
    if (it != g_sms.end()) return it->second;
    int nsm = 0;
    if (cudaDeviceGetAttribute(&nsm, cudaDevAttrMultiProcessorCount, dev) != cudaSuccess || nsm < 1) {
        cudaGetLastError();
        nsm = 1;
    }
    g_sms[dev] = nsm;
    return nsm;
}

int smem_optin() {
    const int dev = current_device();
    std::lock_guard<std::mutex> lock(g_mu);
    auto it = g_optin.find(dev);
    if (it != g_optin.end()) return it->second;
    int optin = 0;
    if (cudaDeviceGetAttribute(&optin, cudaDevAttrMaxSharedMemoryPerBlockOptin, dev) != cudaSuccess || optin < 1) {
        cudaGetLastError();
        optin = 227 * 1024;  // GB300's opt-in limit
    }
    g_optin[dev] = optin;
    return optin;
}

int blocks_per_sm(const void* fn, int threads, size_t smem) {
    const int dev = current_device();
    std::lock_guard<std::mutex> lock(g_mu);
    const auto key = std::make_tuple(fn, dev, threads, smem);
    auto it = g_blocks.find(key);
    if (it != g_blocks.end()) return it->second;
    int per = 0;
    if (cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per, fn, threads, smem) != cudaSuccess || per < 1) {
        cudaGetLastError();
        per = 1;
    }
    g_blocks[key] = per;
    return per;
}

}  // namespace gbca
