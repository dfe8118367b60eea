// sweep_life.cu — host side of the bit-sliced Life-like / Larger-than-Life / Generations sweep
// (the kernel and its layout are described in life_kernel.cuh): the rule's comparator tables,
// tile geometry and its cost model, and the dispatch to the per-radius kernels
// (sweep_life_r1.cu .. sweep_life_r7.cu, sweep_life_vn1.cu .. sweep_life_vn7.cu).
#include "life_common.cuh"

namespace gbca {

namespace {

constexpr double kLifeIoCost = 6.0;   // cell-steps per loaded cell of a pass (the default's cost model)
constexpr double kLifeSatCtas = 2.0;       // CTAs per SM the default's cost model takes to fill an SM,
constexpr double kLifeSatCtasDraws = 3.0;  // and with a Philox gate draw per cell-step

// Intervals of consecutive set bits of a count mask, as intervals of V = count + shift,
// clipped to V <= vmax. Returns false when there are more than kMaxIntervals.
bool intervals(uint64_t mask, int shift, int vmax, int* lo, int* hi, int* n) {
    *n = 0;
    for (int c = 0; c < 64;) {
        if (!((mask >> c) & 1u)) { ++c; continue; }
        int e = c;
        while (e + 1 < 64 && ((mask >> (e + 1)) & 1u)) ++e;
        int a = c + shift, b = e + shift;
        if (b > vmax) b = vmax;
        if (a <= b) {
            if (*n == kMaxIntervals) return false;
            lo[*n] = a;
            hi[*n] = b;
            ++*n;
        }
        c = e + 1;
    }
    return true;
}

bool make_tables(const SweepParams& p, LifeTables* tb) {
    const int N = 2 * p.radius + 1, vmax = N * N;
    int lo[kMaxIntervals], hi[kMaxIntervals], n;
    for (int kind = 0; kind < 2; ++kind) {
        // dead cells: V = count (centre 0), V <= N^2 - 1; live cells: V = count + 1
        if (!intervals(kind == 0 ? p.birth : p.survive, kind, kind == 0 ? vmax - 1 : vmax, lo, hi, &n)) return false;
        tb->n[kind] = n;
        for (int k = 0; k < kMaxIntervals; ++k)
            for (int j = 0; j < 2; ++j) {
                const int L = k < n ? (j == 0 ? lo[k] : hi[k] + 1) : (j == 0 ? 1 : 0);  // unused: empty
                for (int i = 0; i < 8; ++i) tb->m[kind][k][j][i] = ((L >> i) & 1) ? 0u : 0xFFFFFFFFu;
            }
    }
    tb->c3 = p.states > 2 ? 0xFFFFFFFFu : 0u;
    tb->c4 = p.states == 4 ? 0xFFFFFFFFu : 0u;
    for (int i = 0; i < 3; ++i) tb->cb[i] = ((p.states >> i) & 1) ? 0xFFFFFFFFu : 0u;
    return true;
}

// Tile geometry of a pass of K steps; rows = 0 takes the default height.
LifeGeom life_geometry(const SweepParams& p, int K, int rows) {
    LifeGeom g;
    g.K = K;
    g.hy = g.K * p.radius;
    g.hw = (g.hy + 31) / 32;
    const int64_t words = (p.n1 + 31) / 32;
    const int tw = p.tile_x > 0 ? p.tile_x : 32;  // the default choice's width, or 32 words
    g.tw = words < tw ? (int)words : tw;
    const int PL = life_planes(p);
    int ty = PL == 1 ? 216 : (PL == 2 ? 96 : 64);  // more planes: fewer rows
    if (rows > 0) ty = rows;
    g.ty = p.n2 < ty ? (int)p.n2 : ty;
    g.sw = g.tw + 2 * g.hw + 2;
    g.sy = g.ty + 2 * g.hy;
    return g;
}

}  // namespace

size_t life_smem_bytes(const SweepParams& p, const LifeGeom& g) {
    const int PL = life_planes(p);
    const int planes = 2 * PL + (p.mask ? 1 : 0);  // two buffers of PL planes, and the mask's bits
    return (size_t)planes * (size_t)g.sw * (size_t)g.sy * 4;
}

namespace {

// The kernel of the problem's rule, neighbourhood and radius (life_simd_supported holds).
cudaError_t launch_by_rule(const SweepParams& p, const LifeGeom& g, const LifeTables& tb, const int8_t* src,
                           int8_t* dst, cudaStream_t st, int ntiles) {
    if (p.nbhd == GBCA_VON_NEUMANN) {  // radius 1..7
        switch (p.radius) {
            case 1: return launch_life_vn<1>(p, g, tb, src, dst, st, ntiles);
            case 2: return launch_life_vn<2>(p, g, tb, src, dst, st, ntiles);
            case 3: return launch_life_vn<3>(p, g, tb, src, dst, st, ntiles);
            case 4: return launch_life_vn<4>(p, g, tb, src, dst, st, ntiles);
            case 5: return launch_life_vn<5>(p, g, tb, src, dst, st, ntiles);
            case 6: return launch_life_vn<6>(p, g, tb, src, dst, st, ntiles);
            default: return launch_life_vn<7>(p, g, tb, src, dst, st, ntiles);
        }
    }
    switch (p.radius) {
        case 1: return launch_life_radius<1>(p, g, tb, src, dst, st, ntiles);
        case 2: return launch_life_radius<2>(p, g, tb, src, dst, st, ntiles);
        case 3: return launch_life_radius<3>(p, g, tb, src, dst, st, ntiles);
        case 4: return launch_life_radius<4>(p, g, tb, src, dst, st, ntiles);
        case 5: return launch_life_radius<5>(p, g, tb, src, dst, st, ntiles);
        case 6: return launch_life_radius<6>(p, g, tb, src, dst, st, ntiles);
        default: return launch_life_radius<7>(p, g, tb, src, dst, st, ntiles);
    }
}

}  // namespace

bool life_simd_supported(const SweepParams& p) {
    if (p.radius < 1 || p.pitch % 16 != 0) return false;
    if (p.mask && (((uintptr_t)p.mask & 15u) != 0 || p.radius > 5)) return false;  // the gated kernels: r <= 5
    if (p.nbhd != GBCA_MOORE && p.nbhd != GBCA_VON_NEUMANN) return false;
    if (p.scheme == GBCA_CHECKERBOARD) {
        // any boundary: the gate maps halo cells to the cells they image (checker_gate)
    } else if (p.scheme == GBCA_STOCHASTIC) {
        if (p.n1 * p.n2g >= ((int64_t)1 << 32) - 1) return false;  // gate ids in the draws' 32-bit form
    } else if (p.scheme != GBCA_SYNCHRONOUS) {
        return false;
    }
    if (p.scheme != GBCA_SYNCHRONOUS && p.radius > 5) return false;  // gated kernels: r <= 5
    // a closed or masked Life cell keeps its value: the indicator bits hold it only for 0 and 1
    if ((p.scheme != GBCA_SYNCHRONOUS || p.mask) && p.rule == GBCA_RULE_LIFE && !p.states_valid) return false;
    if (p.rule == GBCA_RULE_LIFE) {
        if (p.radius > 7) return false;  // counts up to 15^2 = 225 in 8 bit planes
    } else if (p.rule == GBCA_RULE_GENERATIONS) {
        // two planes hold states 0..3, three 0..7; every state (and Constant value) must lie in 0..C-1;
        // Moore(1, 2) and von Neumann(1..3)
        if (p.radius > (p.nbhd == GBCA_VON_NEUMANN ? 3 : 2) || p.states > 8 || !p.states_valid) return false;
        for (int a = 0; a < 2; ++a)
            if (p.bnd[a] == GBCA_CONSTANT && (p.cval[a] < 0 || p.cval[a] >= p.states)) return false;
    } else {
        return false;
    }
    LifeTables tb;
    return make_tables(p, &tb);
}

// Default steps per pass by radius (the halo grows by r per step).
int life_steps_per_pass(const SweepParams& p) {
    switch (p.radius) {
        case 1: return 16;
        case 2: return 8;
        case 3: return 6;
        case 4: return 5;
        default: return 4;
    }
}

// The geometry for a lattice that has no tuned or pinned one: the steps per pass, tile height
// and tile width that minimise a cost model of one pass per cell-update. A pass costs the
// busiest SM's CTAs (ceil(CTAs / SMs), at least kLifeSatCtas: one 8-warp CTA does not keep an
// SM busy) times the work of one CTA, at a per-SM rate, plus a fixed launch cost. A CTA's
// work is the cells it computes — its tile plus the halo each sub-step recomputes, ex = (K - 1 - s) r rows on each side and one word on each side while
// ex > 0 — plus its loaded region (tile and full halo) at kLifeIoCost cell-steps per cell for
// packing bytes into bits and unpacking the results; that term favours deep passes. Wide tiles
// and deep passes waste least on large lattices; narrower, shorter tiles fill the GPU on
// medium ones (a 2048^2 lattice has 20 CTAs of 1024 x 216 cells). kLifeIoCost = 6 fits the
// measured rates of Life B3/S23 on a 16384^2 torus at 16 and at 4 steps per pass (8.5 and
// 5.0 Tcell-updates/s at 1024 x 216-cell tiles).
SweepChoice life_default_choice(const SweepParams& p0) {
    SweepParams p = p0;
    const int Kmax = life_steps_per_pass(p);
    const int PL = life_planes(p);
    // seconds per SM: a cell-step of the bit-sliced rule, plus a Philox gate draw per cell-step
    // under Stochastic (about 3.3e9 draws per second per SM), and a loaded cell's packing
    const double rate = 60e9 / (p.radius * PL);
    const double c_step = 1.0 / rate + (p.scheme == GBCA_STOCHASTIC ? 1.0 / 3.3e9 : 0.0);
    const double c_io = kLifeIoCost / rate;
    // CTAs an SM needs to reach that rate: more when each cell-step waits on a draw's long chain
    const double sat = p.scheme == GBCA_STOCHASTIC ? kLifeSatCtasDraws : kLifeSatCtas;
    const double t_launch = 4e-6;
    const int nsm = device_sms();
    const int optin = smem_optin();
    const int64_t words = (p.n1 + 31) / 32;
    SweepChoice best = {Kmax, 0, 0};
    double best_cost = -1.0;
    const int Ks[3] = {Kmax, Kmax / 2, Kmax / 4};
    const int tws[3] = {32, 16, 8};
    const int tys[5] = {216, 128, 96, 64, 32};
    for (int K : Ks) {
        if (K < 1) continue;
        for (int tw : tws) {
            const int twe = words < tw ? (int)words : tw;
            if (twe < tw && tw != tws[0] && words < tws[0]) continue;  // narrower than the lattice already
            for (int ty : tys) {
                const int tye = p.n2 < ty ? (int)p.n2 : ty;
                p.tile_x = twe;
                const int KS = K * p.ngates;  // sub-steps (two half-steps per Checkerboard step)
                const LifeGeom g = life_geometry(p, KS, tye);
                if (life_smem_bytes(p, g) > (size_t)optin) continue;
                const int64_t ctas = ((words + twe - 1) / twe) * ((p.n2 + tye - 1) / tye);
                double steps = 0.0;  // cell-steps of one CTA over the pass
                for (int s = 0; s < KS; ++s) {
                    const int ex = (KS - 1 - s) * p.radius;
                    steps += 32.0 * (twe + 2 * ((ex + 31) / 32)) * (tye + 2 * ex);
                }
                const double loaded = 32.0 * (twe + 2 * g.hw) * (tye + 2 * g.hy);
                // an SM reaches its rate with about kLifeSatCtas CTAs resident: fewer leave it idle
                const double per_sm = (double)((ctas + nsm - 1) / nsm);
                const double t = (per_sm > sat ? per_sm : sat) * (steps * c_step + loaded * c_io) + t_launch;
                const double cost = t / ((double)p.n1 * (double)p.n2 * K);
                if (best_cost < 0.0 || cost < best_cost) {
                    best_cost = cost;
                    best = SweepChoice{K, tye, 0};
                    best.tile_words = twe;
                }
            }
        }
    }
    return best;
}

bool life_choice_fits(const SweepParams& p, int steps, int rows) {
    if (steps < 1 || rows < 1) return false;
    const int optin = smem_optin();
    return life_smem_bytes(p, life_geometry(p, steps * p.ngates, rows)) <= (size_t)optin;
}

cudaError_t launch_life_simd(const SweepParams& p0, const int8_t* src, int8_t* dst, cudaStream_t st) {
    SweepParams p = p0;
    if (p.scheme == GBCA_STOCHASTIC) p.keys = philox_keys(p.seed);  // the gate draws
    LifeTables tb;
    if (!make_tables(p, &tb)) return cudaErrorNotSupported;
    LifeGeom g = life_geometry(p, p.nsub, p.tile_y);  // tile_y: the autotuner's pick, or 0
    if (p.mask) {  // the mask's plane: a pick made for the unmasked rule may need shorter tiles
        const int optin = smem_optin();
        for (int ty = g.ty; life_smem_bytes(p, g) > (size_t)optin && ty > 8;) {
            ty /= 2;
            g = life_geometry(p, p.nsub, ty);
        }
    }
    return launch_by_rule(p, g, tb, src, dst, st, 0);
}

}  // namespace gbca

namespace gbca {

cudaError_t launch_life_tiles(const SweepParams& p0, const SparseTiles& sp, const int8_t* src, int8_t* dst,
                              cudaStream_t st) {
    SweepParams p = p0;
    if (p.scheme == GBCA_STOCHASTIC) p.keys = philox_keys(p.seed);  // the gate draws
    LifeTables tb;
    if (!make_tables(p, &tb)) return cudaErrorNotSupported;
    LifeGeom g;
    g.K = p.nsub;
    g.hy = g.K * p.radius;
    g.hw = (g.hy + 31) / 32;
    g.tw = sp.tile_w / 32;
    g.ty = sp.tile_h;
    g.sw = g.tw + 2 * g.hw + 2;
    g.sy = g.ty + 2 * g.hy;
    return launch_by_rule(p, g, tb, src, dst, st, sp.tiles_x * sp.tiles_y);
}

}  // namespace gbca