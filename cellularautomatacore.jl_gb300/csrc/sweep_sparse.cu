// sweep_sparse.cu — active-tile scheduling, the GPU form of the reference's SparseBackend
// (src/sparse.jl): for a quiescent rule (a background cell with background neighbours stays
// background, sparse.jl:42-63) only the tiles holding a non-background cell, and the tiles
// within reach of them, need a sweep (sparse.jl:130-149); every other tile stays background.
//
// The state stays dense in HBM. A flag per tile and per state buffer records whether the tile
// holds a non-background cell. Before each temporally blocked pass, one kernel lists the
// candidate tiles: those within reach (the pass's halo, in tiles, plus one for a partial last
// tile under periodic wrap) of a flagged tile of the source buffer, those flagged in the
// destination buffer (their stale contents must be overwritten), and the tiles along a
// Constant edge whose value is not the background (sparse.jl:103-110). Then one CTA per listed
// tile runs the pass and writes the tile's new flag: the bit-sliced kernel for the Life-like and
// Generations rules it supports, else the general kernel. Tiles never listed keep background
// in both buffers, so results equal the dense sweep's cell for cell.
#include "gbca_internal.cuh"

namespace gbca {

namespace {

__global__ void k_candidates(const uint8_t* __restrict__ flags_src, const uint8_t* __restrict__ flags_dst,
                             int tiles_x, int tiles_y, int reach_x, int reach_y, int wrap_x, int wrap_y, int edge_x,
                             int edge_y, int32_t* __restrict__ list, int32_t* __restrict__ count) {
    const int n = tiles_x * tiles_y;
    for (int tile = blockIdx.x * blockDim.x + threadIdx.x; tile < n; tile += gridDim.x * blockDim.x) {
        const int tx = tile % tiles_x, ty = tile / tiles_x;
        bool cand = flags_dst[tile] != 0;
        cand |= edge_x && (tx < reach_x || tx >= tiles_x - reach_x);
        cand |= edge_y && (ty < reach_y || ty >= tiles_y - reach_y);
        for (int dy = -reach_y; dy <= reach_y && !cand; ++dy) {
            int y = ty + dy;
            if (y < 0 || y >= tiles_y) {
                if (!wrap_y) continue;
                y = (y % tiles_y + tiles_y) % tiles_y;
            }
            for (int dx = -reach_x; dx <= reach_x; ++dx) {
                int x = tx + dx;
                if (x < 0 || x >= tiles_x) {
                    if (!wrap_x) continue;
                    x = (x % tiles_x + tiles_x) % tiles_x;
                }
                if (flags_src[y * tiles_x + x]) {
                    cand = true;
                    break;
                }
            }
        }
        if (cand) list[atomicAdd(count, 1)] = tile;
    }
}

// flags[tile] = the tile holds a cell other than the background.
__global__ void k_tile_flags(const int8_t* __restrict__ u, int64_t n1, int64_t n2, int64_t pitch, int tile_w,
                             int tile_h, int tiles_x, int8_t background, uint8_t* __restrict__ flags) {
    const int tile = blockIdx.x;
    const int64_t X0 = (int64_t)(tile % tiles_x) * tile_w, Y0 = (int64_t)(tile / tiles_x) * tile_h;
    int any = 0;
    for (int q = threadIdx.x; q < tile_w * tile_h; q += blockDim.x) {
        const int64_t x = X0 + q % tile_w, y = Y0 + q / tile_w;
        if (x < n1 && y < n2) any |= u[x + y * pitch] != background;
    }
    any = __syncthreads_or(any);
    if (threadIdx.x == 0) flags[tile] = (uint8_t)any;
}

}  // namespace

cudaError_t launch_candidates(const SweepParams& p, const SparseTiles& sp, int cur, int halo, cudaStream_t st) {
    // the pass reads `halo` cells around a tile: that many tiles, plus one for a partial last
    // tile under periodic wrap
    const int reach_x = (halo + sp.tile_w - 1) / sp.tile_w + 1, reach_y = (halo + sp.tile_h - 1) / sp.tile_h + 1;
    cudaError_t e = cudaMemsetAsync(sp.count, 0, sizeof(int32_t), st);
    if (e != cudaSuccess) return e;
    const int n = sp.tiles_x * sp.tiles_y;
    const int edge_x = p.bnd[0] == GBCA_CONSTANT && p.cval[0] != sp.background;
    const int edge_y = p.bnd[1] == GBCA_CONSTANT && p.cval[1] != sp.background;
    const int blocks = (n + 255) / 256 < 4096 ? (n + 255) / 256 : 4096;
    k_candidates<<<blocks, 256, 0, st>>>(sp.flags[cur], sp.flags[cur ^ 1], sp.tiles_x, sp.tiles_y, reach_x,
                                         reach_y, p.bnd[0] == GBCA_PERIODIC, p.bnd[1] == GBCA_PERIODIC, edge_x, edge_y,
                                         sp.list, sp.count);
    count_launch();
    return cudaGetLastError();
}

cudaError_t launch_tile_flags(const int8_t* u, int64_t n1, int64_t n2, int64_t pitch, const SparseTiles& sp,
                              uint8_t* flags, cudaStream_t st) {
    k_tile_flags<<<sp.tiles_x * sp.tiles_y, 256, 0, st>>>(u, n1, n2, pitch, sp.tile_w, sp.tile_h, sp.tiles_x,
                                                          (int8_t)sp.background, flags);
    count_launch();
    return cudaGetLastError();
}

// The rule evaluated at a background cell whose neighbours are all background: src/rules.jl:385-389
// (Life), :446-456 (Generations), the forest fire of README.md:56-60 (its draws can only fire
// when p > 0 for an empty cell, f > 0 for a tree).
bool rule_quiescent(const gbca_desc& d, const double* params, int32_t bg) {
    const int r = d.radius;
    const int M = d.nbhd == GBCA_MOORE ? (2 * r + 1) * (2 * r + 1) - 1 : 2 * r * (r + 1);
    const int n = bg == 1 ? M : 0;  // neighbours equal to 1
    auto bit = [](uint64_t m, int k) { return k < 64 && ((m >> k) & 1u); };
    switch (d.rule) {
        case GBCA_RULE_LIFE: {
            const int next = bit(bg == 1 ? d.survive : d.birth, n) ? 1 : 0;
            return next == bg;
        }
        case GBCA_RULE_GENERATIONS: {
            if (bg == 0) return !bit(d.birth, n);
            if (bg == 1) return bit(d.survive, n);
            return false;  // s >= 2 always moves on
        }
        case GBCA_RULE_FOREST_FIRE: {
            if (!params) return false;
            if (bg == 2) return false;
            const double p = bg == 0 ? params[0] : params[1];
            return !(d.params_f32 ? (float)p > 0.0f : p > 0.0);
        }
        default:
            return false;
    }
}

}  // namespace gbca
