// fire_words.cuh — one forest-fire sub-step over a region of a shared Int8 tile, four cells
// (one 32-bit word) per work item: the neighbour tests in byte SIMD from five aligned shared
// loads, then four independent Philox4x32-10 draws keyed as src/random.jl:102-107.
// Shared by the single-lattice kernel (sweep_fire.cu) and the batched engine (ensemble.cu).
#pragma once

#include "gbca_internal.cuh"

namespace gbca {

// Bytes equal to `pattern`'s byte -> bit 7 of that byte set (exact: no carries cross bytes).
__device__ __forceinline__ uint32_t bytes_eq(uint32_t x, uint32_t pattern) {
    const uint32_t z = x ^ pattern;
    return ~(((z & 0x7F7F7F7Fu) + 0x7F7F7F7Fu) | z) & 0x80808080u;
}

// The lattice facts one sub-step needs.
struct FireGeom {
    int64_t n1, n2;
    int32_t bnd0, bnd1;
    uint32_t cst0, cst1;   // Constant value of each axis, replicated in every byte
    // thresholds against a draw's raw words (w.x:w.y): Ua + k dU for draw index k (mod 2^64),
    // which is Up for k = 1 (an empty cell) and Uf for k = 2 (a tree)
    uint64_t Ua, dU;
    uint32_t allp, allf;   // 0x01010101 if p >= 1 (resp. f >= 1: every draw hits), else 0
    bool exact_always;     // a Constant edge holds a value other than 0, 1, 2
    int64_t col0, n2g;     // the lattice as a slab of a larger one (SweepParams::col0, n2g)
};

// The global column of local lattice column my (0 <= my < n2): the column of its cells' ids
// and Checkerboard parities.
__device__ __forceinline__ int64_t fire_gcol(const FireGeom& g, int64_t my) {
    int64_t c = my + g.col0;
    if (c < 0) c += g.n2g;
    else if (c >= g.n2g) c -= g.n2g;
    return c;
}

// Whether a Constant edge value is one the bit tests cannot read (anything but 0, 1, 2).
__host__ __device__ inline bool fire_odd_constant(int32_t b0, int32_t c0, int32_t b1, int32_t c1) {
    return (b0 == GBCA_CONSTANT && (c0 < 0 || c0 > 2)) || (b1 == GBCA_CONSTANT && (c1 < 0 || c1 > 2));
}

// Thresholds of bernoulli(p) against the raw words as one 64-bit compare: for a Float64 p,
// (w.x:w.y) >> 11 < T is (w.x:w.y) < T * 2^11; for a Float32 p, (w.x >> 8) < T is
// w.x < T * 2^8, which is (w.x:w.y) < T * 2^40 whatever w.y. A threshold at or above the
// scale (p >= 1) hits always: flagged, since T * 2^11 or T * 2^40 would not fit.
__host__ __device__ inline void fire_thresholds(uint64_t thr_p, uint64_t thr_f, bool f32, FireGeom& g) {
    const uint64_t full = f32 ? ((uint64_t)1 << 24) : ((uint64_t)1 << 53);
    const int shift = f32 ? 40 : 11;
    const bool all_p = thr_p >= full, all_f = thr_f >= full;
    g.allp = all_p ? 0x01010101u : 0u;
    g.allf = all_f ? 0x01010101u : 0u;
    const uint64_t Up = all_p ? 0 : thr_p << shift, Uf = all_f ? 0 : thr_f << shift;
    g.dU = Uf - Up;
    g.Ua = Up - g.dU;
}

// Whether a draw with index k falls below its cell's threshold: bernoulli(p) for an empty cell
// (k = 1), bernoulli(f) for a tree (k = 2), without a branch, so the four draws of a word
// interleave. The threshold Ua + k dU is formed by integer multiply-adds rather than selects:
// the sweep's limit is the ALU pipe (the Philox XORs and the rule's byte logic), and the
// multiply-adds issue to the FMA pipe beside it. A saturated p or f (>= 1) is applied per
// word (fire_next).
__device__ __forceinline__ bool fire_below(uint2 w, uint32_t k, const FireGeom& g) {
    uint64_t t;
    uint32_t hi;
    asm("mad.wide.u32 %0, %1, %2, %3;" : "=l"(t) : "r"(k), "r"((uint32_t)g.dU), "l"(g.Ua));
    asm("mad.lo.u32 %0, %1, %2, %3;" : "=r"(hi) : "r"(k), "r"((uint32_t)(g.dU >> 32)), "r"((uint32_t)(t >> 32)));
    const uint64_t U = ((uint64_t)hi << 32) | (uint32_t)t;
    const uint64_t x = ((uint64_t)w.x << 32) | (uint64_t)w.y;
    return x < U;
}

// Byte masks of a word of four cells (bit 0 of byte b for cell b): empty, tree, and next to a
// burning cell, from the word C and its neighbour words (Lf, Rt: the cells left and right;
// Up, Dn: the rows above and below). EXACT compares whole bytes, for tiles that may hold
// states other than 0, 1, 2 (other values are trees); otherwise a tree is bit 0, a fire bit 1
// and an empty cell neither bit.
template <bool EXACT>
__device__ __forceinline__ void fire_masks(uint32_t C, uint32_t Lf, uint32_t Rt, uint32_t Up, uint32_t Dn,
                                           uint32_t& E, uint32_t& T, uint32_t& N) {
    if (!EXACT) {
        E = ~(C | (C >> 1)) & 0x01010101u;
        T = C & 0x01010101u;
        N = ((Lf | Rt | Up | Dn) >> 1) & 0x01010101u;
    } else {
        E = bytes_eq(C, 0u) >> 7;
        T = ~(E | (bytes_eq(C, 0x02020202u) >> 7)) & 0x01010101u;
        N = (bytes_eq(Lf, 0x02020202u) | bytes_eq(Rt, 0x02020202u) | bytes_eq(Up, 0x02020202u) |
             bytes_eq(Dn, 0x02020202u)) >> 7;
    }
}

// The next states of a word of four cells from its byte masks: cell b (id base + mx[b]) draws
// once, k = 1 if empty else 2; empty -> 1 on a hit, fire -> 0, tree -> 2 next to a fire or on a
// hit, else 1. Byte arithmetic throughout, each cell's code in its own byte: the next state is
// T + (T & (N | H)) + (E & H), no byte above 2, so no carry crosses a byte.
__device__ __forceinline__ uint32_t fire_next(uint32_t E, uint32_t T, uint32_t N, uint32_t base, const uint32_t* mx,
                                              const FireGeom& g, const DrawStep& ds, const PhiloxKeys& K) {
    // hits: a saturated probability hits every cell of its kind (byte select of allp / allf)
    uint32_t H = (E & g.allp) | (~E & g.allf);
    const uint32_t Kw = 0x02020202u - E;  // byte b: cell b's draw index, 1 if empty else 2
#pragma unroll
    for (int b = 0; b < 4; ++b) {
        const uint32_t k = __byte_perm(Kw, 0u, 0x4440u | b);
        const uint2 w = draw_fast(ds, K, base + mx[b], k);
        if (fire_below(w, k, g)) H |= 1u << (8 * b);
    }
    return T + (T & (N | H)) + (E & H);
}

// Words [w_lo, w_lo + nw) x rows [y_lo, y_lo + nrows) of a tile with row pitch sw words; byte
// b of word w in row ly is the cell at lattice (gx0 + 4w + b, gy0 + ly) before mapping. With
// MAPPED the positions go through the boundary map (cells beyond a Constant edge keep the
// constant); without it every position is a lattice cell. A and B must hold a word before
// w_lo and after w_lo + nw - 1 in every row used, and a row above and below.
// `exact` (uniform) compares whole bytes, for tiles that may hold states other than 0, 1, 2
// (a state the caller wrote); otherwise the tests read bits 0 and 1 only. A step of the rule
// only produces 0, 1 and 2, so only the first step after a write needs `exact`.
template <bool MAPPED, bool EXACT>
__device__ __forceinline__ void fire_substep_words_t(const uint32_t* __restrict__ A, uint32_t* __restrict__ B, int sw,
                                                     int w_lo, int nw, int y_lo, int nrows, int64_t gx0, int64_t gy0,
                                                     const FireGeom& g, const DrawStep& ds, const PhiloxKeys& K,
                                                     int tid, int nthr) {
    const uint32_t n1 = (uint32_t)g.n1;
    // (word, row) of this thread's first item, and the stride of nthr items, without a
    // division per item
    const int dlw = nthr % nw, dly = nthr / nw;
    int cw = tid % nw, cy = tid / nw;
    for (int it = tid; it < nw * nrows; it += nthr) {
        const int lw = w_lo + cw, ly = y_lo + cy;
        cw += dlw;
        cy += dly;
        if (cw >= nw) {
            cw -= nw;
            ++cy;
        }
        const int o = ly * sw + lw;
        const uint32_t C = A[o], Wl = A[o - 1], Wr = A[o + 1], Up = A[o - sw], Dn = A[o + sw];
        const uint32_t Lf = __funnelshift_l(Wl, C, 8);  // byte b = cell x - 1
        const uint32_t Rt = __funnelshift_r(C, Wr, 8);  // byte b = cell x + 1
        uint32_t E, T, N;
        fire_masks<EXACT>(C, Lf, Rt, Up, Dn, E, T, N);
        const int64_t gy = gy0 + ly, gx = gx0 + 4 * lw;
        uint32_t outmask = 0, my = (uint32_t)gy;
        uint32_t mx[4];
        bool rowout = false;
        if (MAPPED) {
            const int64_t m = map_axis(g.bnd1, gy, g.n2);
            rowout = m < 0;
            my = (uint32_t)m;
#pragma unroll
            for (int b = 0; b < 4; ++b) {
                const int64_t mb = map_axis(g.bnd0, gx + b, g.n1);
                mx[b] = (uint32_t)mb;
                if (mb < 0) outmask |= 0xFFu << (8 * b);
            }
        } else {
#pragma unroll
            for (int b = 0; b < 4; ++b) mx[b] = (uint32_t)gx + b;
        }
        const uint32_t gc = (uint32_t)fire_gcol(g, rowout ? 0 : (int64_t)my);
        uint32_t res = fire_next(E, T, N, gc * n1 + 1u, mx, g, ds, K);
        if (MAPPED) {
            if (rowout) res = g.cst1;
            else res = (res & ~outmask) | (g.cst0 & outmask);
        }
        B[o] = res;
    }
}

// `exact` (uniform) compares whole bytes, for tiles that may hold states other than 0, 1, 2
// (a state the caller wrote); otherwise the tests read bits 0 and 1 only. A step of the rule
// only produces 0, 1 and 2, so only the first step after a write needs `exact`.
template <bool MAPPED>
__device__ __forceinline__ void fire_substep_words(const uint32_t* __restrict__ A, uint32_t* __restrict__ B, int sw,
                                                   int w_lo, int nw, int y_lo, int nrows, int64_t gx0, int64_t gy0,
                                                   const FireGeom& g, const DrawStep& ds, const PhiloxKeys& K,
                                                   int tid, int nthr, bool exact) {
    if (exact || g.exact_always)
        fire_substep_words_t<MAPPED, true>(A, B, sw, w_lo, nw, y_lo, nrows, gx0, gy0, g, ds, K, tid, nthr);
    else
        fire_substep_words_t<MAPPED, false>(A, B, sw, w_lo, nw, y_lo, nrows, gx0, gy0, g, ds, K, tid, nthr);
}

// The same sub-step with threads on word columns, for an output region of lattice cells whose
// results go straight to the lattice state (gdst, pitch gpitch bytes between columns): thread
// t takes column w_lo + t % nw and a contiguous run of rows (the rows split into nthr / nw
// runs), walking down it so each row reuses the two row words it loaded for the row above (3
// shared loads per word instead of 5) and steps its address and cell ids by one row. Needs
// nw <= nthr; threads past the last whole run stay idle. Every word's first cell lies inside
// the lattice; with CHECKED the last word of a row may reach past column n1, and only its
// cells inside are stored.
// A one-step sweep's gate and mask (src/schemes.jl:84-93, src/environment.jl:123-130): a closed
// or masked cell keeps its state. mode 0: every cell updates; 1: Checkerboard half-step `gate`
// (cells with (x + y) even for gate 0, odd for gate 1); 2: Stochastic, a cell opens when its draw
// k = 0 falls below the raw threshold Ug (or always, allg). mask: nonzero bytes update (pitch
// mpitch between columns), or null.
struct FireGate {
    int32_t mode, gate;
    uint64_t Ug;
    bool allg;
    const uint8_t* mask;
    int64_t mpitch;
};

// Bytes of w that are nonzero, as 0xFF bytes.
__device__ __forceinline__ uint32_t bytes_nonzero(uint32_t w) {
    const uint32_t hi = (w | ((w & 0x7F7F7F7Fu) + 0x7F7F7F7Fu)) & 0x80808080u;
    return (hi >> 7) * 0xFFu;
}

// ROWS: rows of the walk unrolled together (2 lets the row words rotate without moves: 415.5
// against 407.5 Gcell-updates/s on a 16384^2 one-step sweep; the batched kernel, at its
// 64-register cap, keeps 1).
template <bool CHECKED, bool EXACT, bool GATED, int ROWS>
__device__ __forceinline__ void fire_substep_rows_t(const uint32_t* __restrict__ A, int sw, int w_lo, int nw, int y_lo,
                                                    int nrows, int64_t gx0, int64_t gy0, const FireGeom& g,
                                                    const DrawStep& ds, const PhiloxKeys& K, int tid, int nthr,
                                                    int8_t* __restrict__ gdst, int64_t gpitch, const FireGate* fg) {
    const int nseg = nthr / nw, seg = tid / nw;
    if (seg >= nseg) return;
    const int r0 = y_lo + (int)(((int64_t)seg * nrows) / nseg), r1 = y_lo + (int)(((int64_t)(seg + 1) * nrows) / nseg);
    if (r0 >= r1) return;
    const int lw = w_lo + tid % nw;
    const uint32_t n1 = (uint32_t)g.n1;
    const int64_t gx = gx0 + 4 * lw;
    // the column's cells (a cell past n1 is drawn with an id of its own and never stored)
    uint32_t mx[4];
#pragma unroll
    for (int b = 0; b < 4; ++b) mx[b] = (uint32_t)gx + b;
    int o = r0 * sw + lw;
    uint32_t Up = A[o - sw], C = A[o];
    int64_t gy = gy0 + r0;
    int64_t gg = fire_gcol(g, gy);            // the row's global column
    uint32_t base = (uint32_t)gg * n1 + 1u;  // id of the row's cell 0
    int8_t* q = gdst + gx + gy * gpitch;
    const int64_t xin = g.n1 - gx;  // cells of this word inside the lattice (>= 1)
    int ly = r0;
    while (ly < r1) {
        // the rows before the global column wraps to 0 (all of them but on a slab of a torus whose
        // halo crosses the lattice's edge), ids stepped by n1 a row
        const int seg_end = (int64_t)(r1 - ly) <= g.n2g - gg ? r1 : ly + (int)(g.n2g - gg);
#pragma unroll (ROWS)
        for (; ly < seg_end; ++ly, o += sw, q += gpitch, ++gy, ++gg, base += n1) {
            const uint32_t Dn = A[o + sw], Wl = A[o - 1], Wr = A[o + 1];
            const uint32_t Lf = __funnelshift_l(Wl, C, 8);  // byte b = cell x - 1
            const uint32_t Rt = __funnelshift_r(C, Wr, 8);  // byte b = cell x + 1
            uint32_t E, T, N;
            fire_masks<EXACT>(C, Lf, Rt, Up, Dn, E, T, N);
            uint32_t res = fire_next(E, T, N, base, mx, g, ds, K);
            if constexpr (GATED) {  // open bytes take the rule's state, closed and masked ones keep theirs
                uint32_t Gb = 0xFFFFFFFFu;
                if (fg->mode == 1) {
                    Gb = ((gg + fg->gate) & 1) ? 0xFF00FF00u : 0x00FF00FFu;  // gx is even
                } else if (fg->mode == 2 && !fg->allg) {
                    Gb = 0u;
#pragma unroll
                    for (int b = 0; b < 4; ++b) {
                        const uint2 w = draw_fast(ds, K, base + mx[b], 0u);
                        if ((((uint64_t)w.x << 32) | (uint64_t)w.y) < fg->Ug) Gb |= 0xFFu << (8 * b);
                    }
                }
                if (fg->mask) Gb &= bytes_nonzero(*(const uint32_t*)(fg->mask + gx + gy * fg->mpitch));
                res = (res & Gb) | (C & ~Gb);
            }
            if (!CHECKED || xin >= 4) {
                *(uint32_t*)q = res;
            } else {
                for (int b = 0; b < xin; ++b) q[b] = (int8_t)(res >> (8 * b));
            }
            Up = C;
            C = Dn;
        }
        gg = 0;  // the next row is global column 0
        base = 1u;
    }
}

// GATED: the sweep has a gate or a mask (fg), compiled apart from the synchronous, unmasked one.
template <bool CHECKED, bool GATED = false, int ROWS = 1>
__device__ __forceinline__ void fire_substep_rows(const uint32_t* __restrict__ A, int sw, int w_lo, int nw, int y_lo,
                                                  int nrows, int64_t gx0, int64_t gy0, const FireGeom& g,
                                                  const DrawStep& ds, const PhiloxKeys& K, int tid, int nthr,
                                                  bool exact, int8_t* __restrict__ gdst, int64_t gpitch,
                                                  const FireGate* fg = nullptr) {
    if (exact || g.exact_always)
        fire_substep_rows_t<CHECKED, true, GATED, ROWS>(A, sw, w_lo, nw, y_lo, nrows, gx0, gy0, g, ds, K, tid, nthr,
                                                        gdst, gpitch, fg);
    else
        fire_substep_rows_t<CHECKED, false, GATED, ROWS>(A, sw, w_lo, nw, y_lo, nrows, gx0, gy0, g, ds, K, tid, nthr,
                                                         gdst, gpitch, fg);
}

// The gate of a one-step sweep from its parameters (gate = the sub-step's half, 0 or 1), and
// whether the sweep has one.
__device__ __forceinline__ bool fire_gate(int32_t scheme, int32_t gate, uint64_t gate_thr, int32_t gate_f32,
                                          const uint8_t* mask, int64_t pitch, FireGate& fg) {
    fg.mode = scheme == GBCA_CHECKERBOARD ? 1 : (scheme == GBCA_STOCHASTIC ? 2 : 0);
    fg.gate = gate;
    // bernoulli(p) of the gate draw against its raw words, as fire_thresholds does for p and f
    fg.allg = gate_f32 ? gate_thr >= ((uint64_t)1 << 24) : gate_thr >= ((uint64_t)1 << 53);
    fg.Ug = fg.allg ? 0 : gate_thr << (gate_f32 ? 40 : 11);
    fg.mask = mask;
    fg.mpitch = pitch;
    return fg.mode != 0 || mask != nullptr;
}

}  // namespace gbca
