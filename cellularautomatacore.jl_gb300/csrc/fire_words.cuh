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

// Bit 0 of each of 4 bytes -> bits 0..3.
__device__ __forceinline__ uint32_t gather4(uint32_t m01) { return (m01 * 0x10204080u) >> 28; }

// Bits 0..3 -> bit 0 of each of 4 bytes.
__device__ __forceinline__ uint32_t spread4(uint32_t m) { return ((m & 0xFu) * 0x00204081u) & 0x01010101u; }

// The lattice facts one sub-step needs.
struct FireGeom {
    int64_t n1, n2;
    int32_t bnd0, bnd1;
    uint32_t cst0, cst1;   // Constant value of each axis, replicated in every byte
    uint64_t Up, Uf;       // thresholds scaled to the raw Philox words
    bool all_p, all_f;     // p >= 1, f >= 1 (every draw hits)
    bool f32;
    bool exact_always;     // a Constant edge holds a value other than 0, 1, 2
};

// Whether a Constant edge value is one the bit tests cannot read (anything but 0, 1, 2).
__host__ __device__ inline bool fire_odd_constant(int32_t b0, int32_t c0, int32_t b1, int32_t c1) {
    return (b0 == GBCA_CONSTANT && (c0 < 0 || c0 > 2)) || (b1 == GBCA_CONSTANT && (c1 < 0 || c1 > 2));
}

// Thresholds of bernoulli(p) against the raw words: (w.x:w.y) >> 11 < T is
// (w.x:w.y) < T * 2^11 (Float64 p); (w.x >> 8) < T is w.x < T * 2^8 (Float32 p).
__host__ __device__ inline void fire_thresholds(uint64_t thr_p, uint64_t thr_f, bool f32, FireGeom& g) {
    g.f32 = f32;
    g.all_p = !f32 && thr_p >= ((uint64_t)1 << 53);
    g.all_f = !f32 && thr_f >= ((uint64_t)1 << 53);
    g.Up = f32 ? (thr_p << 8) : (g.all_p ? 0 : thr_p << 11);
    g.Uf = f32 ? (thr_f << 8) : (g.all_f ? 0 : thr_f << 11);
}

__device__ __forceinline__ bool fire_hit(uint2 w, bool empty, const FireGeom& g) {
    if (empty ? g.all_p : g.all_f) return true;
    const uint64_t U = empty ? g.Up : g.Uf;
    if (g.f32) return (uint64_t)w.x < U;
    return ((((uint64_t)w.x) << 32) | (uint64_t)w.y) < U;
}

// Words [w_lo, w_lo + nw) x rows [y_lo, y_lo + nrows) of a tile with row pitch sw words; byte
// b of word w in row ly is the cell at lattice (gx0 + 4w + b, gy0 + ly) before mapping. With
// MAPPED the positions go through the boundary map (cells beyond a Constant edge keep the
// constant); without it every position is a lattice cell. A and B must hold a word before
// w_lo and after w_lo + nw - 1 in every row used, and a row above and below.
// `exact` (uniform) compares whole bytes, for tiles that may hold states other than 0, 1, 2
// (a state the caller wrote); otherwise the tests read bits 0 and 1 only. A step of the rule
// only produces 0, 1 and 2, so only the first step after a write needs `exact`.
template <bool MAPPED>
__device__ __forceinline__ void fire_substep_words(const uint32_t* __restrict__ A, uint32_t* __restrict__ B, int sw,
                                                   int w_lo, int nw, int y_lo, int nrows, int64_t gx0, int64_t gy0,
                                                   const FireGeom& g, const DrawStep& ds, const PhiloxKeys& K,
                                                   int tid, int nthr, bool exact) {
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
        // 4-bit masks (bit b = cell b of the word): empty, burning, a burning neighbour
        uint32_t E4, F4, N4;
        if (!exact && !g.exact_always) {
            // every state in {0, 1, 2}: == 2 is bit 1, == 0 is neither bit
            E4 = gather4(~(C | (C >> 1)) & 0x01010101u);
            F4 = gather4((C >> 1) & 0x01010101u);
            N4 = gather4(((Lf | Rt | Up | Dn) >> 1) & 0x01010101u);
        } else {  // any Int8 value (other values are trees): exact byte compares
            E4 = gather4(bytes_eq(C, 0u) >> 7);
            F4 = gather4(bytes_eq(C, 0x02020202u) >> 7);
            N4 = gather4((bytes_eq(Lf, 0x02020202u) | bytes_eq(Rt, 0x02020202u) | bytes_eq(Up, 0x02020202u) |
                          bytes_eq(Dn, 0x02020202u)) >> 7);
        }
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
        const uint32_t base = my * n1 + 1u;
        uint2 w[4];
#pragma unroll
        for (int b = 0; b < 4; ++b) w[b] = draw_fast(ds, K, base + mx[b], 2u - ((E4 >> b) & 1u));
        uint32_t H4 = 0;
#pragma unroll
        for (int b = 0; b < 4; ++b) H4 |= (uint32_t)fire_hit(w[b], (E4 >> b) & 1u, g) << b;
        // next states: empty -> 1 on a hit; fire -> 0; tree -> 2 next to a fire or on a hit, else 1
        const uint32_t T4 = ~(E4 | F4) & 0xFu;
        const uint32_t one = (E4 & H4) | (T4 & ~(N4 | H4)), two = T4 & (N4 | H4);
        uint32_t res = spread4(one) | (spread4(two) << 1);
        if (MAPPED) {
            if (rowout) res = g.cst1;
            else res = (res & ~outmask) | (g.cst0 & outmask);
        }
        B[o] = res;
    }
}

// The same sub-step with threads on word columns: thread t takes column w_lo + t % nw and
// a contiguous run of rows (the rows split into nthr / nw runs), walking down it so each row
// reuses the two row words it loaded for the row above (3 shared loads per word instead of
// 5) and steps its addresses and cell ids by one row each. Needs nw <= nthr; threads past
// the last whole run stay idle. With gdst set (a sweep's last sub-step, whose region is the
// output tile), results go straight to the lattice state (pitch bytes between columns), only
// the cells inside the lattice, instead of to B.
template <bool MAPPED>
__device__ __forceinline__ void fire_substep_rows(const uint32_t* __restrict__ A, uint32_t* __restrict__ B, int sw,
                                                  int w_lo, int nw, int y_lo, int nrows, int64_t gx0, int64_t gy0,
                                                  const FireGeom& g, const DrawStep& ds, const PhiloxKeys& K, int tid,
                                                  int nthr, bool exact, int8_t* __restrict__ gdst = nullptr,
                                                  int64_t gpitch = 0) {
    const int nseg = nthr / nw, seg = tid / nw;
    if (seg >= nseg) return;
    const int r0 = y_lo + (int)(((int64_t)seg * nrows) / nseg), r1 = y_lo + (int)(((int64_t)(seg + 1) * nrows) / nseg);
    if (r0 >= r1) return;
    const int lw = w_lo + tid % nw;
    const uint32_t n1 = (uint32_t)g.n1;
    const int64_t gx = gx0 + 4 * lw;
    // the column's cells: their lattice x (mapped) and which lie beyond a Constant edge
    uint32_t mx[4];
    uint32_t xout = 0;
#pragma unroll
    for (int b = 0; b < 4; ++b) {
        if (MAPPED) {
            const int64_t mb = map_axis(g.bnd0, gx + b, g.n1);
            mx[b] = (uint32_t)mb;
            if (mb < 0) xout |= 0xFFu << (8 * b);
        } else {
            mx[b] = (uint32_t)gx + b;
        }
    }
    int o = r0 * sw + lw;
    uint32_t Up = A[o - sw], C = A[o];
    int64_t gy = gy0 + r0;
    // direct stores: the column's first cell and how many of its 4 cells lie inside the lattice
    int8_t* q = gdst ? gdst + gx + gy * gpitch : nullptr;
    const int64_t xin = g.n1 - gx;
    for (int ly = r0; ly < r1; ++ly, o += sw, ++gy, q += gpitch) {
        const uint32_t Dn = A[o + sw], Wl = A[o - 1], Wr = A[o + 1];
        const uint32_t Lf = __funnelshift_l(Wl, C, 8);  // byte b = cell x - 1
        const uint32_t Rt = __funnelshift_r(C, Wr, 8);  // byte b = cell x + 1
        uint32_t E4, F4, N4;
        if (!exact && !g.exact_always) {
            E4 = gather4(~(C | (C >> 1)) & 0x01010101u);
            F4 = gather4((C >> 1) & 0x01010101u);
            N4 = gather4(((Lf | Rt | Up | Dn) >> 1) & 0x01010101u);
        } else {
            E4 = gather4(bytes_eq(C, 0u) >> 7);
            F4 = gather4(bytes_eq(C, 0x02020202u) >> 7);
            N4 = gather4((bytes_eq(Lf, 0x02020202u) | bytes_eq(Rt, 0x02020202u) | bytes_eq(Up, 0x02020202u) |
                          bytes_eq(Dn, 0x02020202u)) >> 7);
        }
        uint32_t my = (uint32_t)gy;
        bool rowout = false;
        if (MAPPED) {
            const int64_t m = map_axis(g.bnd1, gy, g.n2);
            rowout = m < 0;
            my = (uint32_t)m;
        }
        const uint32_t base = my * n1 + 1u;
        uint2 w[4];
#pragma unroll
        for (int b = 0; b < 4; ++b) w[b] = draw_fast(ds, K, base + mx[b], 2u - ((E4 >> b) & 1u));
        uint32_t H4 = 0;
#pragma unroll
        for (int b = 0; b < 4; ++b) H4 |= (uint32_t)fire_hit(w[b], (E4 >> b) & 1u, g) << b;
        const uint32_t T4 = ~(E4 | F4) & 0xFu;
        const uint32_t one = (E4 & H4) | (T4 & ~(N4 | H4)), two = T4 & (N4 | H4);
        uint32_t res = spread4(one) | (spread4(two) << 1);
        if (gdst) {  // cells of the output tile: never beyond a lower edge
            if (!MAPPED) {
                *(uint32_t*)q = res;  // an interior tile: every cell is a lattice cell
            } else if (gy < g.n2 && xin > 0) {
                if (xin >= 4) *(uint32_t*)q = res;
                else
                    for (int b = 0; b < xin; ++b) q[b] = (int8_t)(res >> (8 * b));
            }
        } else {
            if (MAPPED) {
                if (rowout) res = g.cst1;
                else res = (res & ~xout) | (g.cst0 & xout);
            }
            B[o] = res;
        }
        Up = C;
        C = Dn;
    }
}

}  // namespace gbca
