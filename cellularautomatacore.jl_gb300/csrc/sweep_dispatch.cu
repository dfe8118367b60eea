// sweep_dispatch.cu — picks the sweep kernel for an Int8 problem and runs nsteps steps as
// temporally blocked passes: the forest-fire kernel (VonNeumann(1), Synchronous), the
// bit-sliced kernel (Life-like on Moore(r <= 7); Generations with C <= 8 on Moore(r <= 2)
// when every state is known to lie in 0..C-1), else the general kernel.
#include <cstring>

#include "gbca_internal.cuh"

namespace gbca {

SweepParams sweep_params(const gbca_desc& d, int64_t pitch, const double* params) {
    SweepParams p;
    std::memset(&p, 0, sizeof p);
    p.n1 = d.n1;
    p.n2 = d.n2;
    p.pitch = pitch;
    for (int a = 0; a < 2; ++a) {
        p.bnd[a] = d.boundary[a];
        p.cval[a] = d.boundary[a] == GBCA_CONSTANT ? (int32_t)d.constant[a] : 0;
    }
    p.rule = d.rule;
    p.nbhd = d.nbhd;
    p.radius = d.radius;
    p.states = d.states;
    p.birth = d.birth;
    p.survive = d.survive;
    p.seed = d.seed;
    p.scheme = d.scheme;
    p.gate_f32 = d.scheme_p_f32;
    p.gate_thr = d.scheme == GBCA_STOCHASTIC ? gbca_threshold(d.scheme_p, d.scheme_p_f32) : 0;
    p.params_f32 = d.params_f32;
    p.ngates = d.scheme == GBCA_CHECKERBOARD ? 2 : 1;
    p.col0 = 0;
    p.n2g = d.n2;
    if (d.rule == GBCA_RULE_FOREST_FIRE && params) {
        p.thr_p = gbca_threshold(params[0], d.params_f32);
        p.thr_f = gbca_threshold(params[1], d.params_f32);
    }
    return p;
}

SweepChoice sweep_choice(const gbca_desc& d, bool fire, bool life, const SweepChoice* force) {
    SweepChoice choice = {0, 0, 0};
    if (force) return *force;
    if ((fire || life) && !tuned_choice(d, &choice) && fire) {
        // untuned forest fire: from 2^22 cells one step per pass, each tile staged by TMA (the
        // compute-bound optimum: 221, 311, 376 and 406 Gcell-updates/s at 2048^2, 4096^2,
        // 8192^2 and 16384^2 on GB300); below, 8 steps per pass with vector loads, an eighth
        // of the launches for a launch-bound grid (156 against 120 at 1024^2)
        choice = d.n1 * d.n2 >= ((int64_t)1 << 22) ? SweepChoice{1, 0, 1} : SweepChoice{8, 0, 0};
    }
    if (life && choice.steps_per_pass == 0) {
        const SweepParams p = sweep_params(d, 0, nullptr);
        if (choice.tile_rows == 0) choice = life_default_choice(p);  // neither tuned nor pinned
        else choice.steps_per_pass = life_steps_per_pass(p);
    }
    return choice;
}

cudaError_t fire_gated_step(SweepParams& p, int8_t* const bufs[2], int* cur, int64_t t, cudaStream_t st) {
    p.nsub = 1;
    p.t0 = t;
    for (int gate = 0; gate < p.ngates; ++gate) {
        p.sub0 = gate;
        const cudaError_t e = launch_fire(p, bufs[*cur], bufs[*cur ^ 1], st);
        if (e != cudaSuccess) return e;
        count_launch();
        *cur ^= 1;
    }
    p.sub0 = 0;
    return cudaSuccess;
}

cudaError_t sweep_int8(const gbca_desc& d, int64_t pitch, int8_t* const bufs[2], int* cur, int64_t t, int64_t nsteps,
                       const double* params, cudaStream_t st, bool states_valid, const SweepChoice* force,
                       const uint8_t* mask, const SparseTiles* sparse, const SlabPlace* slab) {
    SweepParams p = sweep_params(d, pitch, params);
    if (slab) {
        p.col0 = slab->col0;
        p.n2g = slab->n2g;
    }
    p.states_valid = states_valid ? 1 : 0;
    p.mask = mask;
    if (sparse) {  // active tiles only: the bit-sliced kernel where it applies, else the general one
        const int ntiles = sparse->tiles_x * sparse->tiles_y;
        p.tiles_x = sparse->tiles_x;
        p.background = sparse->background;
        p.tile_list = sparse->list;
        p.tile_count = sparse->count;
        const bool life = life_simd_supported(p);
        while (nsteps > 0) {
            int64_t per;
            if (life) {
                per = life_steps_per_pass(p);
                // halo (steps x gates x r) no deeper than half a tile
                const int64_t cap = sparse->tile_h / (2 * p.radius * p.ngates);
                if (per > cap) per = cap > 0 ? cap : 1;
            } else {
                per = kGenericSubsteps / (p.radius * p.ngates);
                if (per < 1) per = 1;
            }
            const int64_t k = nsteps < per ? nsteps : per;
            p.nsub = (int32_t)(k * p.ngates);
            p.t0 = t;
            const int halo = p.nsub * p.radius;
            cudaError_t e = launch_candidates(p, *sparse, *cur, halo, st);
            if (e != cudaSuccess) return e;
            p.flags_out = sparse->flags[*cur ^ 1];
            if (life) {
                e = launch_life_tiles(p, *sparse, bufs[*cur], bufs[*cur ^ 1], st);
            } else {
                p.tile_x = sparse->tile_w;
                p.tile_y = sparse->tile_h;
                p.halo_x = p.halo_y = halo;
                e = launch_generic_tiles(p, ntiles, bufs[*cur], bufs[*cur ^ 1], st);
            }
            if (e != cudaSuccess) return e;
            count_launch();
            *cur ^= 1;
            t += k;
            nsteps -= k;
        }
        return cudaSuccess;
    }
    const bool fire = fire_fast_supported(p);
    const bool life = !fire && life_simd_supported(p);
    const SweepChoice choice = sweep_choice(d, fire, life, force);
    p.tile_y = choice.tile_rows;
    p.staging = choice.staging;
    if (life) p.tile_x = choice.tile_words;
    if (fire && fire_gated(p)) {  // a gate or a mask: one sub-step per launch, states kept as valid as given
        for (; nsteps > 0; ++t, --nsteps) {
            const cudaError_t e = fire_gated_step(p, bufs, cur, t, st);
            if (e != cudaSuccess) return e;
        }
        return cudaSuccess;
    }
    while (nsteps > 0) {
        int64_t k;
        cudaError_t e;
        const int8_t* src = bufs[*cur];
        int8_t* dst = bufs[*cur ^ 1];
        p.t0 = t;
        if (fire) {
            const int64_t per = choice.steps_per_pass > 0 ? choice.steps_per_pass : 8;
            k = nsteps < per ? nsteps : per;
            p.nsub = (int32_t)k;
            e = launch_fire(p, src, dst, st);
            p.states_valid = 1;  // a pass leaves only 0, 1 and 2
        } else if (life) {
            const int64_t per = choice.steps_per_pass > 0 ? choice.steps_per_pass : life_steps_per_pass(p);
            k = nsteps < per ? nsteps : per;
            p.nsub = (int32_t)(k * p.ngates);  // sub-steps: two half-steps per Checkerboard step
            e = launch_life_simd(p, src, dst, st);
        } else {
            int64_t per = kGenericSubsteps / (p.radius * p.ngates);
            if (per < 1) per = 1;
            k = nsteps < per ? nsteps : per;
            p.nsub = (int32_t)(k * p.ngates);
            p.tile_x = p.tile_y = 64;
            p.halo_x = p.halo_y = p.nsub * p.radius;
            e = launch_generic(p, src, dst, st);
        }
        if (e != cudaSuccess) return e;
        count_launch();
        *cur ^= 1;
        t += k;
        nsteps -= k;
    }
    return cudaSuccess;
}

}  // namespace gbca
