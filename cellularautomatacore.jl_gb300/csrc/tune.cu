// tune.cu — the sweep autotuner's candidate geometries and its per-shape cache.
//
// A geometry is (steps per temporally blocked pass, tile height, tile staging). Deeper passes
// re-read HBM less often but redo more halo work; taller tiles cut halo overhead but change how
// many tiles fill the 152 SMs' slots; the forest fire's tiles arrive by vector loads or by one
// TMA copy each. The best pair depends on the lattice size, the radius and
// the rule, so gbca_tune (gbca_api.cu) times the candidates below on the handle's own data and
// stores the fastest here; sweep_int8 then uses it for every later call on that shape (single
// handles and the server's large requests alike). Every geometry gives identical results: a
// geometry only changes which tile computes a cell, never the cell's update.
#include <map>
#include <mutex>
#include <tuple>
#include <vector>

#include "gbca_internal.cuh"

namespace gbca {

namespace {

// rule, neighbourhood, radius, states, n1, n2, boundaries, scheme, device
using ShapeKey = std::tuple<int, int, int, int, int64_t, int64_t, int, int, int, int>;

std::mutex g_mu;
std::map<ShapeKey, SweepChoice> g_cache;

ShapeKey key_of(const gbca_desc& d) {
    int dev = 0;
    cudaGetDevice(&dev);
    return ShapeKey(d.rule, d.nbhd, d.radius, d.states, d.n1, d.n2, d.boundary[0], d.boundary[1], d.scheme, dev);
}

}  // namespace

bool tuned_choice(const gbca_desc& d, SweepChoice* out) {
    std::lock_guard<std::mutex> lock(g_mu);
    auto it = g_cache.find(key_of(d));
    if (it == g_cache.end()) return false;
    *out = it->second;
    return true;
}

void store_choice(const gbca_desc& d, const SweepChoice& c) {
    std::lock_guard<std::mutex> lock(g_mu);
    g_cache[key_of(d)] = c;
}

void forget_choices() {
    std::lock_guard<std::mutex> lock(g_mu);
    g_cache.clear();
}

std::vector<SweepChoice> sweep_candidates(const SweepParams& p) {
    std::vector<SweepChoice> out;
    if (fire_fast_supported(p)) {
        if (fire_gated(p)) {  // one sub-step per launch: only the staging varies
            for (int staging : {0, 1, 2}) out.push_back({1, 0, staging});
            return out;
        }
        // the tile height comes from the launcher's model; the pass depth and the tile staging
        // (vector loads or TMA) vary
        for (int staging : {0, 1})
            for (int k : {1, 2, 3, 4, 6, 8}) out.push_back({k, 0, staging});
        out.push_back({1, 0, 2});  // one step per pass from the persistent prefetching kernel
        return out;
    }
    if (!life_simd_supported(p)) return out;
    static const int kPer[7][5] = {{8, 12, 16, 24, 32}, {4, 6, 8, 12, 16}, {3, 4, 6, 8, 10}, {3, 4, 5, 6, 8},
                                   {2, 3, 4, 5, 6},     {2, 3, 4, 5, 6},   {1, 2, 3, 4, 5}};
    const int* per = kPer[p.radius - 1];
    for (int i = 0; i < 5; ++i)
        for (int ty : {64, 96, 128, 144, 176, 216, 256})
            if (life_choice_fits(p, per[i], ty)) out.push_back({per[i], ty, 0});
    return out;
}

}  // namespace gbca
