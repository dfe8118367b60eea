// life_kernel.cuh — the bit-sliced sweep kernel: Life-like and Larger-than-Life rules
// (src/rules.jl:354-389) on Moore(r) and von Neumann(r), r = 1..7, and Generations
// rules with up to 8 states on Moore(1..2) and von Neumann(1..3), Synchronous, Stochastic(p) or
// Checkerboard and masks (r <= 5), as a bit-sliced, temporally blocked sweep.
//
// Layout. Global memory keeps the user's Int8 column-major state. A CTA stages its tile
// plus a halo of K*r cells in shared memory as ONE BIT PER CELL: bit b of word w of a
// row is the indicator (state == 1) of the cell at x = 32w + b (src/rules.jl:377-383
// counts exactly the neighbours equal to 1, and the next state depends on the centre
// only through the same test, so the indicator is all the dynamics reads). Each row has
// a zero guard word on each side.
//
// Counting. A thread owns a column of 32 cells (one word) and a run of rows. For each
// row it forms the 2r+1 horizontally shifted copies of its word (funnel shifts with the
// neighbour words) and adds them with a full-adder tree into a bit-sliced count Hx
// (2-4 bit planes); a register ring keeps the last 2r+1 Hx rows and a bit-sliced running
// sum V = sum of Hx over rows y-r..y+r is updated by one add and one subtract per row.
// V is the Moore box count including the centre. Von Neumann(1) needs no ring: a row's count
// is its 3-cell horizontal count plus the words above and below; von Neumann(2) and (3) add
// the diamond's 13 or 25 shifted words with the same adder trees.
//
// Rule. A dead cell is born when V lies in one of the birth intervals, a live cell
// survives when V - 1 lies in a survive interval, i.e. V in the interval shifted by one.
// Counts of 64 and more never match (UInt64 masks, rules.jl:388). V >= L for a constant
// L is a chain of majority gates, g = maj(v_i, g, m_i) with m_i = 0 where bit i of L is 1
// and ~0 where it is 0 — one LOP3 per bit with m_i read from the parameter bank.
//
// Generations (src/rules.jl:446-456) with C <= 8 states runs in the same kernel with two bit
// planes per cell for C <= 4 (state = lo + 2 hi) and three for C <= 8 (b0 + 2 b1 + 4 b2): the
// count reads the alive plane (state 1), and the next state is 1 for a born dead cell or a
// surviving live one, 2 for a live cell that does not survive (C > 2), s + 1 for a dying cell
// s >= 2 unless s + 1 == C, which goes to 0 (a three-bit increment compared with C's bits).
// The host guarantees that every state lies in 0..C-1 (it scans the state on the device
// after the user writes it).
//
// Temporal blocking: K sub-steps per HBM pass; the computed region shrinks by r per
// sub-step. Periodic and reflecting halos are images of lattice cells and evolve like
// them; cells beyond a Constant edge are reset to the constant after every sub-step.
//
// Gated schemes (src/schemes.jl:84-93): a sub-step's new bits are blended with the old ones
// through a gate mask, so a closed cell keeps its state. Checkerboard runs two half-steps per
// step, the cells with (x + y) even and then odd (0-based): the mask alternates by bit and row
// inside the lattice, and halo words take the parity of the cells they image (a Reflecting
// edge or a Periodic one of odd length flips it). Stochastic(p) opens cell
// (x, y) when its draw k = 0 at time t falls below p, the draw keyed by the mapped cell's id as
// in the rule's own draws. A closed Life cell keeps its value, which the indicator bits hold
// only for states 0 and 1, so gated Life needs every state in {0, 1} (the host scans it).
//
// Masks (src/environment.jl:123-130) use the gated form too: the loader packs the mask's
// nonzero bytes into one more bit plane, mapped through the boundary like the state, and a
// sub-step's gate is ANDed with it, so a masked cell, and each halo image of one, keeps its
// state.
#pragma once

#include "life_common.cuh"

namespace gbca {

namespace {

// Stochastic draws at the sub-step's time), with the lattice position of local cell 0.
struct LifeGate {
    int32_t mode, gate;
    bool rows_plain;  // Checkerboard: rows need no mapping for their parity (checker_gate)
    int64_t X0, Y0;
    DrawStep ds;
};

// map_axis for an index at most one lattice length beyond an edge (the halo of a pass), without
// a division: one wrap (Periodic) or one reflection; anything farther goes to map_axis.
__device__ __forceinline__ int64_t map_near(int32_t b, int64_t g, int64_t n) {
    if ((uint64_t)g < (uint64_t)n) return g;
    if (b == GBCA_CONSTANT) return -1;
    if (g >= -n && g < 2 * n) {
        if (b == GBCA_PERIODIC) return g < 0 ? g + n : g - n;
        return g < 0 ? -g - 1 : 2 * n - 1 - g;  // Reflecting
    }
    return map_axis(b, g, n);
}

// The Stochastic gate of the 32 cells x = gx .. gx + 31 of lattice row y: bit b open when the
// draw k = 0 of the mapped cell falls below p. Cells beyond a Constant edge get a closed bit
// (the Constant reset overwrites them after the sub-step anyway).
__device__ __forceinline__ uint32_t stochastic_gate(const SweepParams& p, const DrawStep& ds, int64_t gx, int64_t y) {
    uint32_t G = 0;
    const int64_t my = map_near(p.bnd[1], y, p.n2);
    if (my < 0) return 0u;
    const int64_t gy = global_col(p, my);  // the row's global column: its cells' ids
    if (gx >= 0 && gx + 32 <= p.n1) {
        const uint32_t base = (uint32_t)(gx + gy * p.n1) + 1u;
#pragma unroll 4
        for (int b = 0; b < 32; ++b)
            G |= (uint32_t)draw_below(draw_fast(ds, p.keys, base + (uint32_t)b, 0u), p.gate_thr, p.gate_f32 != 0) << b;
        return G;
    }
    if (p.bnd[0] == GBCA_PERIODIC && p.n1 >= 32) {  // a word across the wrap: one modulo, then steps
        int64_t m = gx % p.n1;
        if (m < 0) m += p.n1;
        uint32_t mx = (uint32_t)m;
        const uint32_t row = (uint32_t)(gy * p.n1) + 1u, n1 = (uint32_t)p.n1;
#pragma unroll 4
        for (int b = 0; b < 32; ++b) {
            G |= (uint32_t)draw_below(draw_fast(ds, p.keys, row + mx, 0u), p.gate_thr, p.gate_f32 != 0) << b;
            mx = mx + 1u == n1 ? 0u : mx + 1u;
        }
        return G;
    }
    for (int b = 0; b < 32; ++b) {
        const int64_t mx = map_near(p.bnd[0], gx + b, p.n1);
        if (mx < 0) continue;
        const uint32_t id = (uint32_t)(mx + gy * p.n1) + 1u;
        G |= (uint32_t)draw_below(draw_fast(ds, p.keys, id, 0u), p.gate_thr, p.gate_f32 != 0) << b;
    }
    return G;
}

// The Checkerboard gate of the 32 cells x = gx .. gx + 31 (gx a multiple of 32) of lattice row
// y in half-step `gate`: bit b open when the mapped cell's (x + y) is even for gate 0, odd for
// gate 1 (0-based, as isodd(i + j) with 1-based indices, src/schemes.jl:89). Inside the lattice
// the mask alternates by bit. A cell one lattice length or less beyond an edge images a cell of
// the same parity across a Periodic edge of even length, of the other parity across a Periodic
// edge of odd length or a Reflecting edge (x and -x-1, or 2n-1-x); beyond a Constant edge its
// bit is closed (the cell is reset to the constant after the sub-step). So a word column's gate
// is the alternating mask with fixed bits flipped (`flip`) and cleared (`keep`), set once per
// column; a row only maps its y and picks the mask by parity.
struct CheckerCol {
    uint32_t keep, flip;
    bool exact;  // a lattice narrower than the halo: map cell by cell (checker_gate_exact)
};

__device__ __forceinline__ CheckerCol checker_col(const SweepParams& p, int64_t gx) {
    CheckerCol c{0xFFFFFFFFu, 0u, false};
    if (gx >= 0 && gx + 32 <= p.n1) return c;
    uint32_t out = 0;  // bits of cells beyond either edge
    if (gx < 0) out |= -gx >= 32 ? 0xFFFFFFFFu : ((1u << (int)(-gx)) - 1u);
    if (gx + 32 > p.n1) out |= p.n1 - gx <= 0 ? 0xFFFFFFFFu : (0xFFFFFFFFu << (int)(p.n1 - gx));
    if (p.bnd[0] == GBCA_CONSTANT) c.keep = ~out;
    else if (gx >= -p.n1 && gx + 32 <= 2 * p.n1) c.flip = (p.bnd[0] == GBCA_REFLECTING || (p.n1 & 1)) ? out : 0u;
    else c.exact = true;
    return c;
}

__device__ __noinline__ uint32_t checker_gate_exact(int32_t b0, int64_t n1, int64_t gx, int64_t my, int gate) {
    uint32_t G = 0;
    for (int b = 0; b < 32; ++b) {
        const int64_t mx = map_axis(b0, gx + b, n1);
        if (mx >= 0 && ((mx + my) & 1) == gate) G |= 1u << b;
    }
    return G;
}

// rows_plain: every row images a row of its own parity or lies beyond a Constant edge (axis 2
// Constant, or Periodic of even length), so a row's parity is its own and needs no mapping
// (a lattice of its own only: a slab's rows take their global columns' parities).
__device__ __forceinline__ uint32_t checker_gate(const SweepParams& p, const CheckerCol& c, bool rows_plain,
                                                 int64_t gx, int64_t y, int gate) {
    int64_t my = y;
    if (!rows_plain) {
        my = map_near(p.bnd[1], y, p.n2);
        if (my < 0) return 0u;
        my = global_col(p, my);  // parity of the global column (a slab of a larger lattice)
    }
    if (c.exact) return checker_gate_exact(p.bnd[0], p.n1, gx, my, gate);
    const uint32_t base = ((my + gate) & 1) ? 0xAAAAAAAAu : 0x55555555u;  // gx is even
    return (base ^ c.flip) & c.keep;
}

template <int R>
struct LifeBits {
    static constexpr int N = 2 * R + 1;
    static constexpr int H = N < 4 ? 2 : (N < 8 ? 3 : 4);                        // planes of Hx
    static constexpr int V = N * N < 16 ? 4 : (N * N < 32 ? 5 : (N * N < 64 ? 6 : (N * N < 128 ? 7 : 8)));  // of V
    static_assert(N * N < 256, "the comparator tables hold 8 planes: r <= 7");
};

__device__ __forceinline__ uint32_t maj3(uint32_t a, uint32_t b, uint32_t c) { return (a & b) | (a & c) | (b & c); }

__device__ __forceinline__ void fa(uint32_t a, uint32_t b, uint32_t c, uint32_t& s, uint32_t& k) {
    s = a ^ b ^ c;
    k = maj3(a, b, c);
}

// Bit-sliced count of the 2r+1 words x[0..2r] (full-adder trees, hand-reduced).
template <int R>
__device__ __forceinline__ void hcount(const uint32_t* x, uint32_t* h) {
    if constexpr (R == 1) {
        fa(x[0], x[1], x[2], h[0], h[1]);
    } else if constexpr (R == 2) {
        uint32_t s1, k1, k2;
        fa(x[0], x[1], x[2], s1, k1);
        fa(x[3], x[4], s1, h[0], k2);
        h[1] = k1 ^ k2;
        h[2] = k1 & k2;
    } else if constexpr (R == 3) {
        uint32_t s1, k1, s2, k2, k3;
        fa(x[0], x[1], x[2], s1, k1);
        fa(x[3], x[4], x[5], s2, k2);
        fa(x[6], s1, s2, h[0], k3);
        fa(k1, k2, k3, h[1], h[2]);
    } else if constexpr (R == 4) {
        uint32_t s1, k1, s2, k2, s3, k3, k4, t, m1, m2;
        fa(x[0], x[1], x[2], s1, k1);
        fa(x[3], x[4], x[5], s2, k2);
        fa(x[6], x[7], x[8], s3, k3);
        fa(s1, s2, s3, h[0], k4);
        fa(k1, k2, k3, t, m1);
        h[1] = t ^ k4;
        m2 = t & k4;
        h[2] = m1 ^ m2;
        h[3] = m1 & m2;
    } else if constexpr (R == 5) {
        uint32_t s1, k1, s2, k2, s3, k3, s4, k4, k5, t1, m1, m2;
        fa(x[0], x[1], x[2], s1, k1);
        fa(x[3], x[4], x[5], s2, k2);
        fa(x[6], x[7], x[8], s3, k3);
        fa(x[9], x[10], s1, s4, k4);
        fa(s2, s3, s4, h[0], k5);
        fa(k1, k2, k3, t1, m1);
        fa(k4, k5, t1, h[1], m2);
        h[2] = m1 ^ m2;
        h[3] = m1 & m2;
    } else if constexpr (R == 6) {  // 13 inputs: weight-1 sums, then weight-2 and weight-4 carries
        uint32_t s1, k1, s2, k2, s3, k3, s4, k4, t1, c1, c2, d1, e1, d2, e2, e3;
        fa(x[0], x[1], x[2], s1, k1);
        fa(x[3], x[4], x[5], s2, k2);
        fa(x[6], x[7], x[8], s3, k3);
        fa(x[9], x[10], x[11], s4, k4);
        fa(s1, s2, s3, t1, c1);
        fa(t1, s4, x[12], h[0], c2);
        fa(k1, k2, k3, d1, e1);
        fa(k4, c1, c2, d2, e2);
        h[1] = d1 ^ d2;
        e3 = d1 & d2;
        fa(e1, e2, e3, h[2], h[3]);
    } else {
        static_assert(R == 7, "r = 1..7");
        uint32_t s1, k1, s2, k2, s3, k3, s4, k4, s5, k5, t1, c1, c2, d1, e1, d2, e2, e3;
        fa(x[0], x[1], x[2], s1, k1);
        fa(x[3], x[4], x[5], s2, k2);
        fa(x[6], x[7], x[8], s3, k3);
        fa(x[9], x[10], x[11], s4, k4);
        fa(x[12], x[13], x[14], s5, k5);
        fa(s1, s2, s3, t1, c1);
        fa(t1, s4, s5, h[0], c2);
        fa(k1, k2, k3, d1, e1);
        fa(k4, k5, c1, d2, e2);
        fa(d1, d2, c2, h[1], e3);
        fa(e1, e2, e3, h[2], h[3]);
    }
}

// Hx of one row from the thread's word c and its neighbours l, r.
template <int R>
__device__ __forceinline__ void hrow_words(uint32_t l, uint32_t c, uint32_t r, uint32_t* h) {
    uint32_t x[2 * R + 1];
#pragma unroll
    for (int d = 1; d <= R; ++d) {
        x[R - d] = __funnelshift_l(l, c, d);  // cell x - d
        x[R + d] = __funnelshift_r(c, r, d);  // cell x + d
    }
    x[R] = c;
    hcount<R>(x, h);
}

// Hx of one row: p points at the thread's word of plane 0 (guards make p[-1] and p[1]
// valid); with two or three planes the counted cells are the alive ones (state 1).
template <int R, int PL>
__device__ __forceinline__ void hrow(const uint32_t* p, int ps, uint32_t* h) {
    if constexpr (PL == 1) {
        hrow_words<R>(p[-1], p[0], p[1], h);
    } else if constexpr (PL == 2) {
        hrow_words<R>(p[-1] & ~p[ps - 1], p[0] & ~p[ps], p[1] & ~p[ps + 1], h);
    } else {  // state 1: lo set, both higher planes clear
        hrow_words<R>(p[-1] & ~(p[ps - 1] | p[2 * ps - 1]), p[0] & ~(p[ps] | p[2 * ps]),
                      p[1] & ~(p[ps + 1] | p[2 * ps + 1]), h);
    }
}

template <int BH, int BV>
__device__ __forceinline__ void vadd(uint32_t* v, const uint32_t* h) {
    uint32_t c = v[0] & h[0];
    v[0] ^= h[0];
#pragma unroll
    for (int i = 1; i < BV; ++i) {
        if (i < BH) {
            const uint32_t s = v[i] ^ h[i] ^ c;
            c = maj3(v[i], h[i], c);
            v[i] = s;
        } else {
            const uint32_t s = v[i] ^ c;
            c = v[i] & c;
            v[i] = s;
        }
    }
}

template <int BH, int BV>
__device__ __forceinline__ void vsub(uint32_t* v, const uint32_t* h) {
    uint32_t b = ~v[0] & h[0];
    v[0] ^= h[0];
#pragma unroll
    for (int i = 1; i < BV; ++i) {
        if (i < BH) {
            const uint32_t d = v[i] ^ h[i] ^ b;
            b = maj3(~v[i], h[i], b);
            v[i] = d;
        } else {
            const uint32_t d = v[i] ^ b;
            b = ~v[i] & b;
            v[i] = d;
        }
    }
}

template <int BV>
__device__ __forceinline__ uint32_t ge(const uint32_t* v, const uint32_t* m) {
    uint32_t g = 0xFFFFFFFFu;
#pragma unroll
    for (int i = 0; i < BV; ++i) g = maj3(v[i], g, m[i]);
    return g;
}

// NI interval tests per kind, unrolled; the tables fill unused intervals with an empty one
// (lo = 1, hi + 1 = 0), which never matches. The one- and two-interval forms test every
// interval with no branch; the eight-interval form skips the empty ones by the rule's
// interval counts (a uniform branch), so a three-interval rule pays for three.
template <int BV, int NI>
__device__ __forceinline__ void rule_hits(const uint32_t* v, const LifeTables& tb, uint32_t& dead, uint32_t& live) {
    dead = 0u;
    live = 0u;
#pragma unroll
    for (int k = 0; k < NI; ++k) {
        if (NI <= 2 || k < tb.n[0]) dead |= ge<BV>(v, tb.m[0][k][0]) & ~ge<BV>(v, tb.m[0][k][1]);
        if (NI <= 2 || k < tb.n[1]) live |= ge<BV>(v, tb.m[1][k][0]) & ~ge<BV>(v, tb.m[1][k][1]);
    }
}

// The next state of word column w, row y, from its bit-sliced count v (centre included): the
// rule's birth / survival tests, the gate, and the write to B.
template <int BV, int NI, int PL, bool GATED>
__device__ __forceinline__ void life_emit(const uint32_t* v, const uint32_t* ca, uint32_t* cb, const uint32_t* cm, int y,
                                          int sw, int ps, int w, const LifeTables& tb, const SweepParams& p,
                                          const LifeGate& gt, const CheckerCol& cc) {
    uint32_t dead, live;
    rule_hits<BV, NI>(v, tb, dead, live);
    // the gate: open cells take the rule's state, closed ones keep theirs
    uint32_t G = 0xFFFFFFFFu;
    if constexpr (GATED) {
        if (gt.mode == 1) G = checker_gate(p, cc, gt.rows_plain, gt.X0 + 32 * w, gt.Y0 + y, gt.gate);
        else if (gt.mode == 2) G = stochastic_gate(p, gt.ds, gt.X0 + 32 * w, gt.Y0 + y);
        if (cm) G &= cm[y * sw];  // masked cells keep their state (src/environment.jl:123-130)
    }
    if constexpr (PL == 1) {
        const uint32_t c = ca[y * sw];
        cb[y * sw] = (((c & live) | (~c & dead)) & G) | (c & ~G);
    } else if constexpr (PL == 2) {  // Generations, state = lo + 2 hi
        const uint32_t lo = ca[y * sw], hi = ca[y * sw + ps];
        const uint32_t is0 = ~lo & ~hi, is1 = lo & ~hi, is2 = ~lo & hi;
        cb[y * sw] = (((is0 & dead) | (is1 & live) | (is2 & tb.c4)) & G) | (lo & ~G);
        cb[y * sw + ps] = (((is1 & ~live & tb.c3) | (is2 & tb.c4)) & G) | (hi & ~G);
    } else {  // Generations, state = b0 + 2 b1 + 4 b2 (C <= 8)
        const uint32_t b0 = ca[y * sw], b1 = ca[y * sw + ps], b2 = ca[y * sw + 2 * ps];
        const uint32_t hi = b1 | b2, is0 = ~b0 & ~hi, is1 = b0 & ~hi;
        // a dying cell (s >= 2) moves to s + 1, or to 0 when s + 1 == C (three-bit increment, and
        // C's bits as masks: n == C when no bit differs)
        const uint32_t n0 = ~b0, n1 = b1 ^ b0, n2 = b2 ^ (b1 & b0);
        const uint32_t wrap = ~((n0 ^ tb.cb[0]) | (n1 ^ tb.cb[1]) | (n2 ^ tb.cb[2]));
        const uint32_t dying = hi & ~wrap;
        cb[y * sw] = (((is0 & dead) | (is1 & live) | (dying & n0)) & G) | (b0 & ~G);
        cb[y * sw + ps] = (((is1 & ~live & tb.c3) | (dying & n1)) & G) | (b1 & ~G);
        cb[y * sw + 2 * ps] = ((dying & n2) & G) | (b2 & ~G);
    }
}

// The alive bits of a word (Life: the indicator; Generations: state 1, lo & ~hi [& ~top]).
template <int PL>
__device__ __forceinline__ uint32_t alive_word(const uint32_t* q, int ps) {
    if constexpr (PL == 1) return q[0];
    else if constexpr (PL == 2) return q[0] & ~q[ps];
    else return q[0] & ~(q[ps] | q[2 * ps]);
}

// First input of row offset dy in the von Neumann(R) input list (rows -R..R contribute
// 2(R - |dy|) + 1 horizontally shifted words each).
__host__ __device__ constexpr int vn_base(int R, int dy) {
    int n = 0;
    for (int d = -R; d < dy; ++d) n += 2 * (R - (d < 0 ? -d : d)) + 1;
    return n;
}

// Bit-sliced von Neumann(R) count (centre included) of word column `ca` at row y, R = 2 or 3:
// the diamond's 2R^2 + 2R + 1 shifted alive words (13 or 25) through the full-adder trees of the
// Moore kernel (13 inputs: the 13-input tree; 25: the 15- and 9-input trees, then a ripple add
// with the last input as the carry-in).
template <int R, int PL, int BV>
__device__ __forceinline__ void vn_count(const uint32_t* ca, int y, int sw, int ps, uint32_t* v) {
    static_assert(R == 2 || R == 3, "von Neumann(2) or (3)");
    constexpr int NIN = 2 * R * R + 2 * R + 1;
    uint32_t x[NIN];
#pragma unroll
    for (int dy = -R; dy <= R; ++dy) {
        const uint32_t* row = ca + (y + dy) * sw;
        const uint32_t l = alive_word<PL>(row - 1, ps), c = alive_word<PL>(row, ps), r = alive_word<PL>(row + 1, ps);
        const int k = R - (dy < 0 ? -dy : dy), b = vn_base(R, dy);
        x[b] = c;
#pragma unroll
        for (int d = 1; d <= k; ++d) {
            x[b + 2 * d - 1] = __funnelshift_l(l, c, d);  // cell x - d
            x[b + 2 * d] = __funnelshift_r(c, r, d);      // cell x + d
        }
    }
#pragma unroll
    for (int i = 0; i < BV; ++i) v[i] = 0u;
    if constexpr (R == 2) {
        hcount<6>(x, v);  // 13 inputs, four planes
    } else {
        uint32_t a[4], bb[4], c = x[24];
        hcount<7>(x, a);        // inputs 0..14
        hcount<4>(x + 15, bb);  // inputs 15..23
#pragma unroll
        for (int i = 0; i < 4; ++i) fa(a[i], bb[i], c, v[i], c);
        v[4] = c;
    }
}

// von Neumann(R), R = 4..7, down a column (the diamond of 2R^2 + 2R + 1 cells is too wide for one
// adder tree): the count at row y + 1 is the count at y plus the diamond's lower rim and minus
// its upper rim (the cells one and not the other covers), 2R + 1 cells each:
//   lower rim: rows y + 1 + i at horizontal distance R - i, i = 0..R;
//   upper rim: rows y - R + i at horizontal distance i, i = 0..R.
// vn_rim counts one rim of the step from y to y + 1 (R + 1 rows; one word at distance 0, two
// otherwise).
template <int R, int PL, bool LOWER>
__device__ __forceinline__ void vn_rim(const uint32_t* ca, int y, int sw, int ps, uint32_t* h) {
    uint32_t x[2 * R + 1];
#pragma unroll
    for (int i = 0; i <= R; ++i) {
        const int dy = LOWER ? 1 + i : i - R, d = LOWER ? R - i : i;
        const uint32_t* row = ca + (y + dy) * sw;
        const uint32_t c = alive_word<PL>(row, ps);
        if (d == 0) {
            x[2 * R] = c;
        } else {
            const int j = LOWER ? 2 * i : 2 * (i - 1);  // slots 0 .. 2R - 1 for the pairs
            x[j] = __funnelshift_l(alive_word<PL>(row - 1, ps), c, d);  // cell x - d
            x[j + 1] = __funnelshift_r(c, alive_word<PL>(row + 1, ps), d);  // cell x + d
        }
    }
    hcount<R>(x, h);
}

// The full von Neumann(R) count at row y (centre included): row y + DY's 2 (R - |DY|) + 1 cells
// for DY = -R..R, each row's count added in.
template <int R, int PL, int BV, int DY>
__device__ __forceinline__ void vn_full(const uint32_t* ca, int y, int sw, int ps, uint32_t* v) {
    constexpr int K = R - (DY < 0 ? -DY : DY);
    const uint32_t* row = ca + (y + DY) * sw;
    if constexpr (K == 0) {
        const uint32_t one[1] = {alive_word<PL>(row, ps)};
        vadd<1, BV>(v, one);
    } else {
        uint32_t h[LifeBits<K>::H];
        hrow_words<K>(alive_word<PL>(row - 1, ps), alive_word<PL>(row, ps), alive_word<PL>(row + 1, ps), h);
        vadd<LifeBits<K>::H, BV>(v, h);
    }
    if constexpr (DY < R) vn_full<R, PL, BV, DY + 1>(ca, y, sw, ps, v);
}

// One sub-step of word column w over rows [r0, r1). Moore(R): a ring of the last 2R+1 rows'
// horizontal counts and their running vertical sum. VN, von Neumann(1): each row's count is its
// 3-cell horizontal count plus the cells above and below; von Neumann(2, 3): the diamond's
// shifted words through an adder tree (vn_count); von Neumann(4..7): a running count, the rims
// added and taken away row by row (vn_rim).
template <int R, int NI, int PL, bool GATED, bool VN>
__device__ __forceinline__ void life_column(const uint32_t* __restrict__ A, uint32_t* __restrict__ B,
                                            const uint32_t* __restrict__ M, int sw, int ps, int w, int r0, int r1,
                                            const LifeTables& tb, const SweepParams& p, const LifeGate& gt) {
    constexpr int N = LifeBits<R>::N, BH = LifeBits<R>::H, BV = LifeBits<R>::V;
    const uint32_t* ca = A + 1 + w;
    uint32_t* cb = B + 1 + w;
    const uint32_t* cm = M ? M + 1 + w : nullptr;  // the column's mask bits, or none
    CheckerCol cc{0xFFFFFFFFu, 0u, false};  // the column's Checkerboard mask adjustments
    if constexpr (GATED) {
        if (gt.mode == 1) cc = checker_col(p, gt.X0 + 32 * w);
    }
    if constexpr (VN && R > 3) {
        uint32_t v[BV];
#pragma unroll
        for (int i = 0; i < BV; ++i) v[i] = 0u;
        vn_full<R, PL, BV, -R>(ca, r0, sw, ps, v);
        for (int y = r0; y < r1; ++y) {
            life_emit<BV, NI, PL, GATED>(v, ca, cb, cm, y, sw, ps, w, tb, p, gt, cc);
            if (y + 1 < r1) {
                uint32_t h[BH];
                vn_rim<R, PL, true>(ca, y, sw, ps, h);
                vadd<BH, BV>(v, h);
                vn_rim<R, PL, false>(ca, y, sw, ps, h);
                vsub<BH, BV>(v, h);
            }
        }
    } else if constexpr (VN && R > 1) {
        for (int y = r0; y < r1; ++y) {
            uint32_t v[BV];
            vn_count<R, PL, BV>(ca, y, sw, ps, v);
            life_emit<BV, NI, PL, GATED>(v, ca, cb, cm, y, sw, ps, w, tb, p, gt, cc);
        }
    } else if constexpr (VN) {
        for (int y = r0; y < r1; ++y) {
            uint32_t h[2];
            hrow<1, PL>(ca + y * sw, ps, h);  // cells x - 1, x, x + 1: h0 + 2 h1
            const uint32_t up = alive_word<PL>(ca + (y - 1) * sw, ps), dn = alive_word<PL>(ca + (y + 1) * sw, ps);
            const uint32_t s1 = up ^ dn, c1 = up & dn, k0 = h[0] & s1;
            uint32_t v[BV];
            v[0] = h[0] ^ s1;
            v[1] = h[1] ^ c1 ^ k0;
            v[2] = maj3(h[1], c1, k0);
#pragma unroll
            for (int i = 3; i < BV; ++i) v[i] = 0u;
            life_emit<BV, NI, PL, GATED>(v, ca, cb, cm, y, sw, ps, w, tb, p, gt, cc);
        }
    } else {
        uint32_t ring[N][BH];
        uint32_t v[BV];
#pragma unroll
        for (int i = 0; i < BV; ++i) v[i] = 0u;
#pragma unroll
        for (int k = 0; k < N; ++k) {
            hrow<R, PL>(ca + (r0 - R + k) * sw, ps, ring[k]);
            vadd<BH, BV>(v, ring[k]);
        }
        for (int y0 = r0; y0 < r1; y0 += N) {
#pragma unroll
            for (int k = 0; k < N; ++k) {
                const int y = y0 + k;
                if (y < r1) {
                    life_emit<BV, NI, PL, GATED>(v, ca, cb, cm, y, sw, ps, w, tb, p, gt, cc);
                    if (y + 1 < r1) {
                        vsub<BH, BV>(v, ring[k]);
                        hrow<R, PL>(ca + (y + R + 1) * sw, ps, ring[k]);
                        vadd<BH, BV>(v, ring[k]);
                    }
                }
            }
        }
    }
}
// Indicator bits (byte == 1) of 4 bytes, in bits 0..3.
__device__ __forceinline__ uint32_t ones4(uint32_t w) {
    const uint32_t t = w ^ 0x01010101u;
    const uint32_t nz = ((t & 0x7F7F7F7Fu) + 0x7F7F7F7Fu) | t;
    const uint32_t z = (~nz & 0x80808080u) >> 7;
    return (z * 0x10204080u) >> 28;
}

__device__ __forceinline__ uint32_t ones16(int4 q) {
    return ones4((uint32_t)q.x) | (ones4((uint32_t)q.y) << 4) | (ones4((uint32_t)q.z) << 8) |
           (ones4((uint32_t)q.w) << 12);
}

// Bit `bit` of each of 4 bytes, in bits 0..3 (states 0..3: bit 0 = lo plane, bit 1 = hi).
__device__ __forceinline__ uint32_t plane4(uint32_t w, int bit) {
    return (((w >> bit) & 0x01010101u) * 0x10204080u) >> 28;
}

__device__ __forceinline__ uint32_t plane16(int4 q, int bit) {
    return plane4((uint32_t)q.x, bit) | (plane4((uint32_t)q.y, bit) << 4) | (plane4((uint32_t)q.z, bit) << 8) |
           (plane4((uint32_t)q.w, bit) << 12);
}

// Bits 0..3 of b as four bytes 0/1.
__device__ __forceinline__ uint32_t bytes4(uint32_t b) { return ((b & 0xFu) * 0x00204081u) & 0x01010101u; }

__device__ __forceinline__ int4 bytes16(uint32_t b) {
    return make_int4((int)bytes4(b), (int)bytes4(b >> 4), (int)bytes4(b >> 8), (int)bytes4(b >> 12));
}

// 32 indicator bits of the cells gx .. gx+31 of lattice column-row `row` (already mapped in y).
__device__ __forceinline__ uint32_t load_bits32(const SweepParams& p, const int8_t* __restrict__ row, int64_t gx) {
    int64_t a = -1;
    if (gx >= 0 && gx + 32 <= p.n1) a = gx;
    else if (p.bnd[0] == GBCA_PERIODIC && (p.n1 & 31) == 0) a = map_near(GBCA_PERIODIC, gx, p.n1);
    if (a >= 0) {
        const int4* q = (const int4*)(row + a);
        return ones16(q[0]) | (ones16(q[1]) << 16);
    }
    uint32_t bits = 0;
    for (int b = 0; b < 32; ++b) {
        const int64_t mx = map_near(p.bnd[0], gx + b, p.n1);
        const int v = mx < 0 ? p.cval[0] : row[mx];
        bits |= (uint32_t)(v == 1) << b;
    }
    return bits;
}

// Plane bits (state bit `bit`) of the cells gx .. gx+31 of an already mapped row.
__device__ __forceinline__ uint32_t load_plane32(const SweepParams& p, const int8_t* __restrict__ row, int64_t gx,
                                                 int bit) {
    int64_t a = -1;
    if (gx >= 0 && gx + 32 <= p.n1) a = gx;
    else if (p.bnd[0] == GBCA_PERIODIC && (p.n1 & 31) == 0) a = map_near(GBCA_PERIODIC, gx, p.n1);
    if (a >= 0) {
        const int4* q = (const int4*)(row + a);
        return plane16(q[0], bit) | (plane16(q[1], bit) << 16);
    }
    uint32_t bits = 0;
    for (int b = 0; b < 32; ++b) {
        const int64_t mx = map_near(p.bnd[0], gx + b, p.n1);
        const int v = mx < 0 ? p.cval[0] : row[mx];
        bits |= (uint32_t)((v >> bit) & 1) << b;
    }
    return bits;
}

// Nonzero bytes of 4 bytes, in bits 0..3.
__device__ __forceinline__ uint32_t nonzero4(uint32_t w) {
    const uint32_t hi = (w | ((w & 0x7F7F7F7Fu) + 0x7F7F7F7Fu)) & 0x80808080u;
    return ((hi >> 7) * 0x10204080u) >> 28;
}

__device__ __forceinline__ uint32_t nonzero16(int4 q) {
    return nonzero4((uint32_t)q.x) | (nonzero4((uint32_t)q.y) << 4) | (nonzero4((uint32_t)q.z) << 8) |
           (nonzero4((uint32_t)q.w) << 12);
}

// Mask bits (the cell updates: nonzero byte) of the cells gx .. gx+31 of an already mapped mask
// row; a cell beyond a Constant edge gets 0 (it is reset to the constant anyway).
__device__ __forceinline__ uint32_t load_mask32(const SweepParams& p, const uint8_t* __restrict__ row, int64_t gx) {
    int64_t a = -1;
    if (gx >= 0 && gx + 32 <= p.n1) a = gx;
    else if (p.bnd[0] == GBCA_PERIODIC && (p.n1 & 31) == 0) a = map_near(GBCA_PERIODIC, gx, p.n1);
    if (a >= 0) {
        const int4* q = (const int4*)(row + a);
        return nonzero16(q[0]) | (nonzero16(q[1]) << 16);
    }
    uint32_t bits = 0;
    for (int b = 0; b < 32; ++b) {
        const int64_t mx = map_near(p.bnd[0], gx + b, p.n1);
        if (mx >= 0 && row[mx]) bits |= 1u << b;
    }
    return bits;
}

template <int R, int NI, int PL, bool GATED, bool VN>
__global__ void __launch_bounds__(kLifeThreads) k_life(SweepParams p, LifeGeom g, LifeTables tb,
                                                       const int8_t* __restrict__ src, int8_t* __restrict__ dst) {
    extern __shared__ __align__(16) uint32_t smw[];
    const int ps = g.sw * g.sy;  // words between the planes of one buffer
    uint32_t* A = smw;
    uint32_t* B = smw + PL * ps;
    uint32_t* M = smw + 2 * PL * ps;  // the mask plane (masked sweeps only)
    const int W = g.tw + 2 * g.hw;
    int bx = blockIdx.x, by = blockIdx.y, tile = 0;
    if (p.tile_list) {  // active-tile sweeps: one CTA per listed tile, the rest has nothing to do
        if ((int)blockIdx.x >= *p.tile_count) return;
        tile = p.tile_list[blockIdx.x];
        bx = tile % p.tiles_x;
        by = tile / p.tiles_x;
    }
    const int64_t X0 = (int64_t)bx * (32 * g.tw) - 32 * g.hw;  // lattice x of local cell 0
    const int64_t Y0 = (int64_t)by * g.ty - g.hy;              // lattice y of local row 0
    // the Constant values as plane bits (Life: the indicator; Generations: state bits)
    uint32_t cb0[PL], cb1[PL];
#pragma unroll
    for (int pl = 0; pl < PL; ++pl) {
        cb0[pl] = PL == 1 ? (p.cval[0] == 1 ? 0xFFFFFFFFu : 0u) : (((p.cval[0] >> pl) & 1) ? 0xFFFFFFFFu : 0u);
        cb1[pl] = PL == 1 ? (p.cval[1] == 1 ? 0xFFFFFFFFu : 0u) : (((p.cval[1] >> pl) & 1) ? 0xFFFFFFFFu : 0u);
    }

    for (int q = threadIdx.x; q < W * g.sy; q += blockDim.x) {
        const int lw = q % W, ly = q / W;
        const int64_t my = map_near(p.bnd[1], Y0 + ly, p.n2);
#pragma unroll
        for (int pl = 0; pl < PL; ++pl) {
            uint32_t bits;
            if (my < 0) bits = cb1[pl];
            else if (PL == 1) bits = load_bits32(p, src + my * p.pitch, X0 + 32 * lw);
            else bits = load_plane32(p, src + my * p.pitch, X0 + 32 * lw, pl);
            A[pl * ps + ly * g.sw + 1 + lw] = bits;
            B[pl * ps + ly * g.sw + 1 + lw] = bits;
        }
        if constexpr (GATED) {  // the mask's bits, mapped like the state (a masked cell keeps its state)
            if (p.mask) M[ly * g.sw + 1 + lw] = my < 0 ? 0u : load_mask32(p, p.mask + my * p.pitch, X0 + 32 * lw);
        }
    }
    for (int ly = threadIdx.x; ly < g.sy; ly += blockDim.x) {
#pragma unroll
        for (int pl = 0; pl < PL; ++pl) {
            A[pl * ps + ly * g.sw] = A[pl * ps + ly * g.sw + W + 1] = 0u;
            B[pl * ps + ly * g.sw] = B[pl * ps + ly * g.sw + W + 1] = 0u;
        }
    }
    // does the loaded region reach beyond a Constant edge?
    const bool fix = (p.bnd[0] == GBCA_CONSTANT && (X0 < 0 || X0 + 32 * W > p.n1)) ||
                     (p.bnd[1] == GBCA_CONSTANT && (Y0 < 0 || Y0 + g.sy > p.n2));
    __syncthreads();

    LifeGate gt;  // a gated scheme's sub-step gate (the synchronous kernel has none)
    gt.mode = 0;
    gt.gate = 0;
    gt.rows_plain = (p.col0 == 0 && p.n2g == p.n2) &&
                    (p.bnd[1] == GBCA_CONSTANT || (p.bnd[1] == GBCA_PERIODIC && (p.n2 & 1) == 0));
    gt.X0 = X0;
    gt.Y0 = Y0;
    if constexpr (GATED) gt.mode = p.scheme == GBCA_CHECKERBOARD ? 1 : (p.scheme == GBCA_STOCHASTIC ? 2 : 0);
    for (int s = 0; s < g.K; ++s) {
        if constexpr (GATED) {
            gt.gate = (p.sub0 + s) % p.ngates;
            if (gt.mode == 2) gt.ds = draw_step(p.keys, p.t0 + (p.sub0 + s) / p.ngates);
        }
        const int ex = (g.K - 1 - s) * R;
        const int y_lo = g.hy - ex, y_hi = g.hy + g.ty + ex;
        const int w_lo = (32 * g.hw - ex) >> 5, w_hi = (32 * (g.hw + g.tw) + ex + 31) >> 5;
        const int nw = w_hi - w_lo;
        const int nseg = blockDim.x / nw;
        const int seg = threadIdx.x / nw;
        if (seg < nseg) {
            const int rows = y_hi - y_lo;
            const int r0 = y_lo + (seg * rows) / nseg, r1 = y_lo + ((seg + 1) * rows) / nseg;
            if (r1 > r0)
                life_column<R, NI, PL, GATED, VN>(A, B, GATED && p.mask ? M : nullptr, g.sw, ps,
                                                  w_lo + threadIdx.x % nw, r0, r1, tb, p, gt);
        }
        __syncthreads();
        if (fix) {
            for (int q = threadIdx.x; q < nw * (y_hi - y_lo); q += blockDim.x) {
                const int lw = w_lo + q % nw, ly = y_lo + q / nw;
                const int64_t gy = Y0 + ly, gx = X0 + 32 * lw;
#pragma unroll
                for (int pl = 0; pl < PL; ++pl) {
                    uint32_t* wp = B + pl * ps + ly * g.sw + 1 + lw;
                    if (p.bnd[1] == GBCA_CONSTANT && (gy < 0 || gy >= p.n2)) {
                        *wp = cb1[pl];
                    } else if (p.bnd[0] == GBCA_CONSTANT && (gx < 0 || gx + 32 > p.n1)) {
                        uint32_t out = 0;
                        for (int b = 0; b < 32; ++b) out |= (uint32_t)(gx + b < 0 || gx + b >= p.n1) << b;
                        *wp = (*wp & ~out) | (cb0[pl] & out);
                    }
                }
            }
            __syncthreads();
        }
        uint32_t* t = A; A = B; B = t;
    }

    int active = 0;  // a written cell differs from the background (active-tile sweeps)
    uint32_t bgp[PL];  // the background's plane bits
#pragma unroll
    for (int pl = 0; pl < PL; ++pl) bgp[pl] = ((p.background >> pl) & 1) ? 0xFFFFFFFFu : 0u;
    for (int q = threadIdx.x; q < g.tw * g.ty; q += blockDim.x) {
        const int lw = g.hw + q % g.tw, ly = g.hy + q / g.tw;
        const int64_t gy = Y0 + ly, gx = X0 + 32 * lw;
        if (gy >= p.n2 || gx >= p.n1) continue;
        uint32_t pw[PL];
        uint32_t diff = 0u;
#pragma unroll
        for (int pl = 0; pl < PL; ++pl) {
            pw[pl] = A[pl * ps + ly * g.sw + 1 + lw];
            diff |= pw[pl] ^ bgp[pl];
        }
        const uint32_t valid = gx + 32 <= p.n1 ? 0xFFFFFFFFu : ((1u << (p.n1 - gx)) - 1u);
        active |= (diff & valid) != 0u;
        int8_t* out = dst + gy * p.pitch + gx;
        if (gx + 32 <= p.n1) {
            int4 q0 = bytes16(pw[0]), q1 = bytes16(pw[0] >> 16);
#pragma unroll
            for (int pl = 1; pl < PL; ++pl) {
                const int4 h0 = bytes16(pw[pl]), h1 = bytes16(pw[pl] >> 16);
                q0 = make_int4(q0.x | (h0.x << pl), q0.y | (h0.y << pl), q0.z | (h0.z << pl), q0.w | (h0.w << pl));
                q1 = make_int4(q1.x | (h1.x << pl), q1.y | (h1.y << pl), q1.z | (h1.z << pl), q1.w | (h1.w << pl));
            }
            ((int4*)out)[0] = q0;
            ((int4*)out)[1] = q1;
        } else {
            for (int b = 0; gx + b < p.n1; ++b) {
                uint32_t v = 0;
#pragma unroll
                for (int pl = 0; pl < PL; ++pl) v |= ((pw[pl] >> b) & 1u) << pl;
                out[b] = (int8_t)v;
            }
        }
    }
    if (p.tile_list) {
        active = __syncthreads_or(active);
        if (threadIdx.x == 0) p.flags_out[tile] = (uint8_t)active;
    }
}

template <int R, int NI, int PL, bool GATED, bool VN>
cudaError_t launch_rn(const SweepParams& p, const LifeGeom& g, const LifeTables& tb, const int8_t* src, int8_t* dst,
                      cudaStream_t st, int ntiles) {
    const size_t smem = life_smem_bytes(p, g);
    cudaError_t e = ensure_dynamic_smem((const void*)k_life<R, NI, PL, GATED, VN>, smem);
    if (e != cudaSuccess) return e;
    dim3 grid((unsigned)((p.n1 + 32 * g.tw - 1) / (32 * g.tw)), (unsigned)((p.n2 + g.ty - 1) / g.ty));
    if (ntiles > 0) grid = dim3((unsigned)ntiles, 1u);  // one CTA per listed tile
    k_life<R, NI, PL, GATED, VN><<<grid, kLifeThreads, smem, st>>>(p, g, tb, src, dst);
    return cudaGetLastError();
}

template <int R, int PL, bool VN = false>
cudaError_t launch_r(const SweepParams& p, const LifeGeom& g, const LifeTables& tb, const int8_t* src, int8_t* dst,
                     cudaStream_t st, int ntiles = 0) {
    const int ni = tb.n[0] > tb.n[1] ? tb.n[0] : tb.n[1];
    if (p.scheme != GBCA_SYNCHRONOUS || p.mask) {  // gated variants (gates, masks) exist for r <= 5
        if constexpr (R <= 5) {
            if (ni <= 1) return launch_rn<R, 1, PL, true, VN>(p, g, tb, src, dst, st, ntiles);
            if (ni <= 2) return launch_rn<R, 2, PL, true, VN>(p, g, tb, src, dst, st, ntiles);
            return launch_rn<R, kMaxIntervals, PL, true, VN>(p, g, tb, src, dst, st, ntiles);
        } else {
            return cudaErrorNotSupported;
        }
    }
    if (ni <= 1) return launch_rn<R, 1, PL, false, VN>(p, g, tb, src, dst, st, ntiles);
    if constexpr (R <= 5) {  // radii 6 and 7 compile one- and eight-interval forms only
        if (ni <= 2) return launch_rn<R, 2, PL, false, VN>(p, g, tb, src, dst, st, ntiles);
    }
    return launch_rn<R, kMaxIntervals, PL, false, VN>(p, g, tb, src, dst, st, ntiles);
}


}  // namespace

// Moore(R): Life-like rules, and Generations (two planes up to C = 4, three up to 8) for R <= 2.
template <int R>
cudaError_t launch_life_radius(const SweepParams& p, const LifeGeom& g, const LifeTables& tb, const int8_t* src,
                               int8_t* dst, cudaStream_t st, int ntiles) {
    if constexpr (R <= 2) {
        if (p.rule == GBCA_RULE_GENERATIONS) {
            if (p.states <= 4) return launch_r<R, 2>(p, g, tb, src, dst, st, ntiles);
            return launch_r<R, 3>(p, g, tb, src, dst, st, ntiles);
        }
    }
    return launch_r<R, 1>(p, g, tb, src, dst, st, ntiles);
}

// von Neumann(R): Life-like rules, and Generations (two or three planes) for R <= 3.
template <int R>
cudaError_t launch_life_vn(const SweepParams& p, const LifeGeom& g, const LifeTables& tb, const int8_t* src,
                           int8_t* dst, cudaStream_t st, int ntiles) {
    if constexpr (R <= 3) {
        if (p.rule == GBCA_RULE_GENERATIONS) {
            if (p.states <= 4) return launch_r<R, 2, true>(p, g, tb, src, dst, st, ntiles);
            return launch_r<R, 3, true>(p, g, tb, src, dst, st, ntiles);
        }
    }
    return launch_r<R, 1, true>(p, g, tb, src, dst, st, ntiles);
}

}  // namespace gbca
