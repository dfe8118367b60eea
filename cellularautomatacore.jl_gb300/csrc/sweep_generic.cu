// sweep_generic.cu — the general temporally blocked Int8 sweep: every supported rule
// (Life / Larger-than-Life, Generations, forest fire), Moore and von Neumann
// neighbourhoods of any radius, every boundary kind and every gated scheme
// (Synchronous, Stochastic(p), Checkerboard).
//
// One CTA owns an output tile. It stages the tile plus a halo of nsub*r cells in shared
// memory, read through the boundary mapping (the halo of src/backends.jl:425-442 is
// folded into this loader), then runs nsub sub-steps in shared memory, each one the
// per-cell update of src/backends.jl:444-455 over a region that shrinks by r per
// sub-step, and writes the tile once. Cells of the halo that are periodic or reflected
// images of lattice cells are updated with the id (hence the draws and the checkerboard
// parity) of the cell they image; cells beyond a Constant edge keep the constant. Masked
// cells (src/environment.jl:123-130) keep their state, images included.
#include "gbca_internal.cuh"

namespace gbca {

namespace {

// RC: the radius when it is known at compile time (1, the common neighbourhoods, whose loops
// then unroll), 0 to read it from p.
template <int RC>
__device__ __forceinline__ int8_t generic_rule(const SweepParams& p, const int8_t* A, int sx, int lx, int ly,
                                               int8_t c, uint64_t id, int64_t t) {
    const int r = RC > 0 ? RC : p.radius;
    int n = 0;
    bool fire = false;
    if (p.nbhd == GBCA_MOORE) {
        for (int dj = -r; dj <= r; ++dj) {
            const int8_t* row = A + (ly + dj) * sx + lx;
            for (int di = -r; di <= r; ++di) {
                if (di == 0 && dj == 0) continue;
                const int8_t v = row[di];
                n += (v == 1);
                fire |= (v == 2);
            }
        }
    } else {
        for (int dj = -r; dj <= r; ++dj) {
            const int8_t* row = A + (ly + dj) * sx + lx;
            const int rr = r - (dj < 0 ? -dj : dj);
            for (int di = -rr; di <= rr; ++di) {
                if (di == 0 && dj == 0) continue;
                const int8_t v = row[di];
                n += (v == 1);
                fire |= (v == 2);
            }
        }
    }
    if (p.rule == GBCA_RULE_LIFE) {  // src/rules.jl:385-389
        const uint64_t mask = c == 1 ? p.survive : p.birth;
        return (int8_t)(n < 64 ? (mask >> n) & 1u : 0u);
    }
    if (p.rule == GBCA_RULE_GENERATIONS) {  // src/rules.jl:446-456
        const int s = c;
        if (s == 0) return (int8_t)(n < 64 ? (p.birth >> n) & 1u : 0u);
        if (s == 1) {
            if (n < 64 && ((p.survive >> n) & 1u)) return c;
            return (int8_t)(p.states > 2 ? 2 : 0);
        }
        return (int8_t)(s + 1 < p.states ? s + 1 : 0);
    }
    // forest fire (README.md:56-60 on Int8 codes): 2 -> 0; 0 -> 1 w.p. p (draw 1);
    // otherwise 2 next to a fire, else 2 w.p. f (draw 2), else 1.
    if (c == 2) return 0;
    if (c == 0) return draw_below(cell_draw(p.seed, id, t, 1), p.thr_p, p.params_f32) ? 1 : 0;
    if (fire) return 2;
    return draw_below(cell_draw(p.seed, id, t, 2), p.thr_f, p.params_f32) ? 2 : 1;
}

template <bool TILES, int RC>
__global__ void __launch_bounds__(256) k_generic(SweepParams p, const int8_t* __restrict__ src,
                                                 int8_t* __restrict__ dst) {
    extern __shared__ int8_t smem_g[];
    const int hx = p.halo_x, hy = p.halo_y;
    const int sx = p.tile_x + 2 * hx, sy = p.tile_y + 2 * hy;
    int8_t* A = smem_g;
    int8_t* B = smem_g + sx * sy;
    int64_t X0, Y0;
    int tile = 0;
    if (TILES) {  // one CTA per listed tile; the rest of the grid has nothing to do
        if ((int)blockIdx.x >= *p.tile_count) return;
        tile = p.tile_list[blockIdx.x];
        X0 = (int64_t)(tile % p.tiles_x) * p.tile_x;
        Y0 = (int64_t)(tile / p.tiles_x) * p.tile_y;
    } else {
        X0 = (int64_t)blockIdx.x * p.tile_x;
        Y0 = (int64_t)blockIdx.y * p.tile_y;
    }
    const bool interior = X0 - hx >= 0 && X0 + p.tile_x + hx <= p.n1 && Y0 - hy >= 0 &&
                          Y0 + p.tile_y + hy <= p.n2;

    // rows to warps, cells of a row to lanes: no division per cell
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5, nwarps = blockDim.x >> 5;
    for (int ly = warp; ly < sy; ly += nwarps) {
        const int64_t gy = Y0 - hy + ly;
        const int64_t my = interior ? gy : map_axis(p.bnd[1], gy, p.n2);
        for (int lx = lane; lx < sx; lx += 32) {
            const int64_t gx = X0 - hx + lx;
            int8_t v;
            if (interior) {
                v = src[gx + gy * p.pitch];
            } else {
                const int64_t mx = map_axis(p.bnd[0], gx, p.n1);
                if (my < 0) v = (int8_t)p.cval[1];
                else if (mx < 0) v = (int8_t)p.cval[0];
                else v = src[mx + my * p.pitch];
            }
            A[ly * sx + lx] = v;
        }
    }
    __syncthreads();

    for (int s = 0; s < p.nsub; ++s) {
        const int64_t t = p.t0 + s / p.ngates;
        const int gate = s % p.ngates;
        const int ex = (p.nsub - 1 - s) * p.radius;  // margin still needed after this sub-step
        const int x_lo = hx - ex, y_lo = hy - ex;
        const int w = p.tile_x + 2 * ex, h = p.tile_y + 2 * ex;
        for (int j = warp; j < h; j += nwarps)
        for (int i = lane; i < w; i += 32) {
            const int lx = x_lo + i, ly = y_lo + j;
            int64_t mx = X0 - hx + lx, my = Y0 - hy + ly;
            if (!interior) {
                mx = map_axis(p.bnd[0], mx, p.n1);
                my = map_axis(p.bnd[1], my, p.n2);
                if (mx < 0 || my < 0) {
                    B[ly * sx + lx] = (int8_t)(my < 0 ? p.cval[1] : p.cval[0]);
                    continue;
                }
            }
            const int8_t c = A[ly * sx + lx];
            if (p.mask && !p.mask[mx + my * p.pitch]) {  // a masked cell keeps its state
                B[ly * sx + lx] = c;
                continue;
            }
            const int64_t gc = global_col(p, my);  // the global column: ids and parities
            const uint64_t id = (uint64_t)mx + (uint64_t)gc * (uint64_t)p.n1 + 1u;
            bool open = true;  // src/schemes.jl:84-89
            if (p.scheme == GBCA_STOCHASTIC)
                open = draw_below(cell_draw(p.seed, id, t, 0), p.gate_thr, p.gate_f32);
            else if (p.scheme == GBCA_CHECKERBOARD)
                open = (((mx + gc + 2) & 1) == (gate == 1 ? 1 : 0));
            B[ly * sx + lx] = open ? generic_rule<RC>(p, A, sx, lx, ly, c, id, t) : c;
        }
        __syncthreads();
        int8_t* tmp = A; A = B; B = tmp;
    }

    int active = 0;
    for (int oy = warp; oy < p.tile_y; oy += nwarps)
        for (int ox = lane; ox < p.tile_x; ox += 32) {
            const int64_t gx = X0 + ox, gy = Y0 + oy;
            if (gx < p.n1 && gy < p.n2) {
                const int8_t v = A[(hy + oy) * sx + hx + ox];
                dst[gx + gy * p.pitch] = v;
                if (TILES) active |= v != (int8_t)p.background;
            }
        }
    if (TILES) {
        active = __syncthreads_or(active);
        if (threadIdx.x == 0) p.flags_out[tile] = (uint8_t)active;
    }
}

}  // namespace

namespace {

template <bool TILES>
cudaError_t launch_generic_as(const SweepParams& p, dim3 grid, const int8_t* src, int8_t* dst, cudaStream_t st) {
    const int sx = p.tile_x + 2 * p.halo_x, sy = p.tile_y + 2 * p.halo_y;
    const size_t smem = 2 * (size_t)sx * (size_t)sy;
    void (*fn)(SweepParams, const int8_t*, int8_t*) = p.radius == 1 ? k_generic<TILES, 1> : k_generic<TILES, 0>;
    if (smem > 48 * 1024) {
        cudaError_t e = ensure_dynamic_smem((const void*)fn, smem);
        if (e != cudaSuccess) return e;
    }
    fn<<<grid, 256, smem, st>>>(p, src, dst);
    return cudaGetLastError();
}

}  // namespace

cudaError_t launch_generic(const SweepParams& p, const int8_t* src, int8_t* dst, cudaStream_t st) {
    const dim3 grid((unsigned)((p.n1 + p.tile_x - 1) / p.tile_x), (unsigned)((p.n2 + p.tile_y - 1) / p.tile_y));
    return launch_generic_as<false>(p, grid, src, dst, st);
}

cudaError_t launch_generic_tiles(const SweepParams& p, int ntiles, const int8_t* src, int8_t* dst, cudaStream_t st) {
    return launch_generic_as<true>(p, dim3((unsigned)ntiles), src, dst, st);
}

}  // namespace gbca
