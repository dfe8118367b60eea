// spectral.cu — this library's FFTs for the periodic kernel fields of Lenia and KernelField
// dispersal: U = irfft(rfft(src) .* conj(rfft(kpad))) (ext/CellularAutomataCoreFFTWExt.jl:17-30),
// kpad the kernel's weights wrapped onto the lattice at 0-based (offset mod n) per axis.
//
// Three launches per field, each line of the lattice transformed inside one CTA's shared memory
// by a mixed-radix Stockham FFT (radix 8, 4, 2, 3, 5; self-sorting, so no bit reversal),
// twiddles from per-stage tables computed in FP64 on the host:
//   1. axis 1 (the contiguous axis): two real lines packed as one complex line, transformed,
//      split into the two half spectra (n1/2 + 1 frequencies each), stored as two rows of the
//      work spectrum;
//   2. axis 2, a few axis-1 frequencies a CTA: forward transform, product with the kernel's
//      spectrum (conjugated, with the inverse's 1/(n1 n2) folded in), inverse transform, in place;
//   3. axis 1 inverse: the Hermitian halves of two rows rebuilt into one complex line whose
//      inverse transform holds the two real fields, then the epilogue (Lenia's growth and clamp,
//      or the field stored for the kernel-field sweep); in a run of Lenia steps the same CTA
//      then transforms the new state's two lines (step 1 of the next step).
// Float32 lines of 512, 1024, 2048 or 4096 points take kernels compiled for their length
// (k_pl_*), whose transforms keep their first inputs and last outputs in registers; other
// lengths, and Float64, take the general ones.
// The kernel's spectrum is made once by the same launches in FP64 (steps 1 and 2, forward only).
#include <cmath>
#include <type_traits>
#include <vector>

#include "gbca_internal.cuh"
#include "spectral.cuh"

namespace gbca {

namespace {

template <typename T> struct CxOf;
template <> struct CxOf<float> { using type = float2; };
template <> struct CxOf<double> { using type = double2; };

template <typename C> __device__ __forceinline__ C cadd(C a, C b) { return C{a.x + b.x, a.y + b.y}; }
template <typename C> __device__ __forceinline__ C csub(C a, C b) { return C{a.x - b.x, a.y - b.y}; }
template <typename C> __device__ __forceinline__ C cmul(C a, C b) {
    return C{a.x * b.x - a.y * b.y, a.x * b.y + a.y * b.x};
}
// a * (DIR i): DIR = +1 multiplies by i, -1 by -i
template <int DIR, typename C> __device__ __forceinline__ C cmul_i(C a) {
    return DIR > 0 ? C{-a.y, a.x} : C{a.y, -a.x};
}

constexpr int kMaxStages = 16;
struct FftFactors {
    int n, nst;
    uint64_t code;  // stage s has radix (code >> 4 s) & 15
    __host__ __device__ int radix(int s) const { return (int)((code >> (4 * s)) & 15u); }
};

// n as radices 8, then 4, 2, 3, 5; nst = -1 when n has another prime factor.
FftFactors factorize(int64_t n) {
    FftFactors f;
    f.n = (int)n;
    f.nst = 0;
    f.code = 0;
    int64_t m = n;
    for (int r : {8, 4, 2, 3, 5})
        while (n >= 1 && m % r == 0 && f.nst < kMaxStages) {
            f.code |= (uint64_t)r << (4 * f.nst++);
            m /= r;
        }
    if (m != 1 || n < 1) f.nst = -1;
    return f;
}

// Threads that transform one n-point line: at most 8 points each.
__host__ __device__ inline int line_threads(int n) {
    const int t = (n + 7) / 8;
    return t < 32 ? 32 : (t + 31) / 32 * 32;
}

// The DFT of R points in place (R = 2, 3, 4, 5, 8, 16), exponent sign DIR.
template <int R, int DIR, typename C>
__device__ __forceinline__ void dft_small(C* v) {
    using T = decltype(v[0].x);
    if constexpr (R == 2) {
        const C a = v[0], b = v[1];
        v[0] = cadd(a, b);
        v[1] = csub(a, b);
    } else if constexpr (R == 4) {
        const C a0 = cadd(v[0], v[2]), a1 = csub(v[0], v[2]), a2 = cadd(v[1], v[3]);
        const C a3 = cmul_i<DIR>(csub(v[1], v[3]));
        v[0] = cadd(a0, a2);
        v[1] = cadd(a1, a3);
        v[2] = csub(a0, a2);
        v[3] = csub(a1, a3);
    } else if constexpr (R == 8) {  // two 4-point DFTs (even and odd points) and 4 radix-2 pairs
        C e[4] = {v[0], v[2], v[4], v[6]}, o[4] = {v[1], v[3], v[5], v[7]};
        dft_small<4, DIR>(e);
        dft_small<4, DIR>(o);
        const T r = T(0.70710678118654752440);  // 1 / sqrt(2)
        const C o1 = C{r * (o[1].x - DIR * o[1].y), r * (o[1].y + DIR * o[1].x)};    // (1 + DIR i)/sqrt2 o1
        const C o2 = cmul_i<DIR>(o[2]);                                                  // DIR i o2
        const C o3 = C{r * (-o[3].x - DIR * o[3].y), r * (-o[3].y + DIR * o[3].x)};  // (-1 + DIR i)/sqrt2 o3
        v[0] = cadd(e[0], o[0]);
        v[4] = csub(e[0], o[0]);
        v[1] = cadd(e[1], o1);
        v[5] = csub(e[1], o1);
        v[2] = cadd(e[2], o2);
        v[6] = csub(e[2], o2);
        v[3] = cadd(e[3], o3);
        v[7] = csub(e[3], o3);
    } else if constexpr (R == 3) {
        const T s3 = T(0.86602540378443864676);  // sin(2 pi / 3)
        const C t = cadd(v[1], v[2]);
        const C d = cmul_i<DIR>(csub(v[1], v[2]));
        const C m = C{v[0].x - T(0.5) * t.x, v[0].y - T(0.5) * t.y};
        v[0] = cadd(v[0], t);
        v[1] = C{m.x + s3 * d.x, m.y + s3 * d.y};
        v[2] = C{m.x - s3 * d.x, m.y - s3 * d.y};
    } else if constexpr (R == 16) {  // 4 x 4: DFTs over stride-4 points, twiddles W16^(n2 k1), DFTs across
        C a[4][4];                        // a[n2][k1]
#pragma unroll
        for (int n2 = 0; n2 < 4; ++n2) {
            C w[4] = {v[n2], v[n2 + 4], v[n2 + 8], v[n2 + 12]};
            dft_small<4, DIR>(w);
#pragma unroll
            for (int k1 = 0; k1 < 4; ++k1) a[n2][k1] = w[k1];
        }
        const T c1 = T(0.92387953251128675613), s1 = T(0.38268343236508977173);  // cos, sin(pi / 8)
        const T r = T(0.70710678118654752440);                                   // cos, sin(pi / 4)
        // exp(DIR 2 pi i j / 16) for j = n2 k1: 1 (c1, s1), 2 (r, r), 3 (s1, c1), 4 (0, 1), 6 (-r, r), 9 (-c1, -s1)
        a[1][1] = cmul(a[1][1], C{c1, DIR * s1});
        a[1][2] = cmul(a[1][2], C{r, DIR * r});
        a[1][3] = cmul(a[1][3], C{s1, DIR * c1});
        a[2][1] = cmul(a[2][1], C{r, DIR * r});
        a[2][2] = cmul_i<DIR>(a[2][2]);
        a[2][3] = cmul(a[2][3], C{-r, DIR * r});
        a[3][1] = cmul(a[3][1], C{s1, DIR * c1});
        a[3][2] = cmul(a[3][2], C{-r, DIR * r});
        a[3][3] = cmul(a[3][3], C{-c1, -DIR * s1});
#pragma unroll
        for (int k1 = 0; k1 < 4; ++k1) {
            C w[4] = {a[0][k1], a[1][k1], a[2][k1], a[3][k1]};
            dft_small<4, DIR>(w);
#pragma unroll
            for (int k2 = 0; k2 < 4; ++k2) v[k1 + 4 * k2] = w[k2];
        }
    } else {  // R == 5
        const T c1 = T(0.30901699437494742410), c2 = T(-0.80901699437494742410);  // cos(2 pi / 5), cos(4 pi / 5)
        const T s1 = T(0.95105651629515357212), s2 = T(0.58778525229247312917);   // sin(2 pi / 5), sin(4 pi / 5)
        const C t1 = cadd(v[1], v[4]), t2 = cadd(v[2], v[3]);
        const C d1 = cmul_i<DIR>(csub(v[1], v[4])), d2 = cmul_i<DIR>(csub(v[2], v[3]));
        const C a1 = C{v[0].x + c1 * t1.x + c2 * t2.x, v[0].y + c1 * t1.y + c2 * t2.y};
        const C a2 = C{v[0].x + c2 * t1.x + c1 * t2.x, v[0].y + c2 * t1.y + c1 * t2.y};
        const C b1 = C{s1 * d1.x + s2 * d2.x, s1 * d1.y + s2 * d2.y};
        const C b2 = C{s2 * d1.x - s1 * d2.x, s2 * d1.y - s1 * d2.y};
        v[0] = cadd(v[0], cadd(t1, t2));
        v[1] = cadd(a1, b1);
        v[4] = csub(a1, b1);
        v[2] = cadd(a2, b2);
        v[3] = csub(a2, b2);
    }
}

// Shared-memory slot of point e of a line: one pad slot every 16 points, so that the early
// stages' writes (points 8 apart) and the axis-2 kernel's row loads meet few bank conflicts.
__host__ __device__ __forceinline__ int pad16(int e) { return e + (e >> 4); }
__host__ __device__ inline int padded_len(int n) { return pad16(n - 1) + 1; }

// Twiddles of every stage, stage after stage: for a stage of radix R after sub-transforms of
// length l, W(k, R l)^q = exp(-2 pi i k q / (R l)) at [(q - 1) l + k], q = 1 .. R - 1, k < l:
// consecutive butterflies read consecutive entries. twiddle_count(f) entries in all.
int twiddle_count(const FftFactors& f) {
    int l = 1, c = 0;
    for (int s = 0; s < f.nst; ++s) {
        c += (f.radix(s) - 1) * l;
        l *= f.radix(s);
    }
    return c;
}

// One Stockham stage of radix R with sub-transform length l over the n-point line x (padded
// slots), in place: butterfly j (< n/R) reads points j + q n/R (q < R), turns the inputs by
// W(k, R l)^q with k = j mod l (tw: the stage's table, conjugated for DIR = +1), and writes
// their R-point DFT to points (j - k) R + k + m l. Thread t of the line's T (>= n/8) threads
// takes butterflies t, t + T, ...: at most ceil(8 / R), held in registers between a barrier
// after the reads and the writes, so one buffer serves. Every thread of the CTA must call it
// (two barriers).
template <int R, int DIR, typename C>
__device__ __forceinline__ void fft_stage(C* x, int n, int l, const C* tw, int t, int T) {
    constexpr int B = (8 + R - 1) / R;
    const int nR = n / R;
    const bool l2 = (l & (l - 1)) == 0;
    C v[B][R];
#pragma unroll
    for (int b = 0; b < B; ++b) {
        const int j = t + b * T;
        if (j < nR) {
            const int k = l2 ? (j & (l - 1)) : j % l;
#pragma unroll
            for (int q = 0; q < R; ++q) {
                C a = x[pad16(j + q * nR)];
                if (q > 0) {
                    C w = tw[(q - 1) * l + k];
                    if (DIR > 0) w.y = -w.y;
                    a = cmul(a, w);
                }
                v[b][q] = a;
            }
            dft_small<R, DIR>(v[b]);
        }
    }
    __syncthreads();
#pragma unroll
    for (int b = 0; b < B; ++b) {
        const int j = t + b * T;
        if (j < nR) {
            const int k = l2 ? (j & (l - 1)) : j % l;
            const int base = (j - k) * R + k;
#pragma unroll
            for (int m = 0; m < R; ++m) x[pad16(base + m * l)] = v[b][m];
        }
    }
    __syncthreads();
}

// One line's DFT (exponent sign DIR) in place in shared memory (padded slots), by the line's T
// threads (this thread is t), twiddles from the per-stage table tw (shared memory); every thread
// of the CTA calls it the same number of times. MIX compiles the radix-3 and radix-5 stages too
// (their butterflies hold more registers); without it the line's length is a power of two.
template <int DIR, bool MIX, typename C>
__device__ void fft_line(C* x, const FftFactors& f, const C* tw, int t, int T) {
    int l = 1;
    for (int s = 0; s < f.nst; ++s) {
        const int R = f.radix(s);
        if (R == 8) fft_stage<8, DIR>(x, f.n, l, tw, t, T);
        else if (R == 4) fft_stage<4, DIR>(x, f.n, l, tw, t, T);
        else if (!MIX || R == 2) fft_stage<2, DIR>(x, f.n, l, tw, t, T);
        else if constexpr (MIX) {
            if (R == 3) fft_stage<3, DIR>(x, f.n, l, tw, t, T);
            else fft_stage<5, DIR>(x, f.n, l, tw, t, T);
        }
        tw += (R - 1) * l;
        l *= R;
    }
}

// The per-stage twiddle table into shared memory (by all threads of the CTA; a barrier follows
// before use).
template <typename C>
__device__ __forceinline__ void stage_twiddles(C* dst, const C* __restrict__ src, int count) {
    for (int i = threadIdx.x; i < count; i += blockDim.x) dst[i] = src[i];
}

// Launch bounds of the transform kernels: up to 1024 threads, registers capped at 64 (so two
// 512-thread CTAs share an SM).
constexpr int kFftMaxThreads = 1024;

template <typename T>
__device__ __forceinline__ T load_source(const void* u, int64_t pitch, int x, int64_t y, int src) {
    if (src == kSpecReal) return ((const T*)u)[x + y * pitch];
    const int8_t v = ((const int8_t*)u)[x + y * pitch];
    if (src == kSpecIsOne) return v == 1 ? T(1) : T(0);
    return T(v);
}

// The work spectrum and the kernel's spectrum are stored line by line along axis 2: row y holds
// the axis-1 frequencies k = 0 .. n1/2 of line y, padded to ncp (a multiple of 4) values, so
// that axis-1 kernels read and write whole rows and the axis-2 kernel reads four consecutive
// frequencies of a row as one 32-byte (Float32) piece.
__host__ __device__ inline int spec_pitch(int n1) { return (n1 / 2 + 1 + 3) / 4 * 4; }

// Axis-1 kernels take two real lines (y = 2 b, 2 b + 1) a CTA, as one complex line of n1 points
// transformed by T = line_threads(n1) threads (one such line a CTA ran a Lenia step in 67.9 us
// against 71.9 with two).
constexpr int kAxis1Complex = 1;  // complex lines a CTA
constexpr int kAxis1Lines = 2 * kAxis1Complex;
// The axis-2 kernel takes up to four frequencies a CTA (fewer when four lines would need more
// than kFftMaxThreads threads).
__host__ __device__ inline int axis2_lines(int n2) {
    const int t = line_threads(n2);
    return t * 4 <= kFftMaxThreads ? 4 : (t * 2 <= kFftMaxThreads ? 2 : 1);
}
// Shared-memory stride between the axis-2 kernel's lines: 4 slots (32 bytes in Float32) modulo
// 16, so that one row's four frequencies land in different banks.
__host__ __device__ inline int axis2_line_stride(int n2) { return (padded_len(n2) + 15) / 16 * 16 + 4; }

// A transformed complex line (Z = DFT(line ya + i line ya + 1), padded slots) split into the two
// lines' half spectra, stored as rows ya and ya + 1 of spec (row pitch ncp).
template <typename T, typename C>
__device__ __forceinline__ void split_rows(const C* a, int n1, C* ra, int ncp, bool h0, bool h1, int t, int TL) {
    for (int k = t; k <= n1 / 2; k += TL) {
        const C zk = a[pad16(k)], zm = a[pad16(k == 0 ? 0 : n1 - k)];
        // zc = conj(Z[n1 - k]); Xa = (Zk + zc) / 2, Xb = (Zk - zc) / (2 i)
        if (h0) ra[k] = C{T(0.5) * (zk.x + zm.x), T(0.5) * (zk.y - zm.y)};
        if (h1) ra[ncp + k] = C{T(0.5) * (zk.y + zm.y), T(0.5) * (zm.x - zk.x)};
    }
}

// Step 1: the CTA's lines along axis 1 into rows y of spec.
template <typename T, bool MIX>
__global__ void __launch_bounds__(kFftMaxThreads, 1)
    k_axis1_forward(const void* __restrict__ u, int64_t pitch, int src, int n1, int n2, FftFactors f,
                    const typename CxOf<T>::type* __restrict__ tw, int ntw, typename CxOf<T>::type* __restrict__ spec) {
    using C = typename CxOf<T>::type;
    extern __shared__ __align__(16) unsigned char smem[];
    C* tws = (C*)smem;  // the twiddles, then the two lines
    stage_twiddles(tws, tw, ntw);
    const int TL = line_threads(n1);
    const int li = threadIdx.x / TL, t = threadIdx.x - li * TL;  // the CTA's complex line li
    C* a = tws + ntw + li * padded_len(n1);
    const int64_t ya = (int64_t)kAxis1Lines * blockIdx.x + 2 * li;
    const bool h0 = ya < n2, h1 = ya + 1 < n2;
#pragma unroll 4
    for (int x = t; x < n1; x += TL)
        a[pad16(x)] = C{h0 ? load_source<T>(u, pitch, x, ya, src) : T(0),
                        h1 ? load_source<T>(u, pitch, x, ya + 1, src) : T(0)};
    __syncthreads();
    fft_line<-1, MIX>(a, f, tws, t, TL);
    const int ncp = spec_pitch(n1);
    split_rows<T>(a, n1, spec + ya * ncp, ncp, h0, h1, t, TL);
}

// Step 2: frequencies k0 .. k0 + L - 1 (k0 = L blockIdx.x, L = axis2_lines(n2)) along axis 2,
// line kk by threads kk T .. kk T + T - 1. MUL: forward, times ks, inverse, in place; otherwise
// forward only, into out. Loads and stores go row by row, lanes over the L frequencies first.
template <typename T, bool MUL, bool MIX>
__global__ void __launch_bounds__(kFftMaxThreads, 1) k_axis2(typename CxOf<T>::type* __restrict__ spec,
                                                             const typename CxOf<T>::type* __restrict__ ks,
                                                             typename CxOf<T>::type* __restrict__ out, int n1, int n2,
                                                             FftFactors f, const typename CxOf<T>::type* __restrict__ tw,
                                                             int ntw) {
    using C = typename CxOf<T>::type;
    extern __shared__ __align__(16) unsigned char smem[];
    C* tws = (C*)smem;
    stage_twiddles(tws, tw, ntw);
    C* lines = tws + ntw;  // line kk at lines + kk LP
    const int L = axis2_lines(n2), TL = line_threads(n2), ncp = spec_pitch(n1), nc = n1 / 2 + 1;
    const int LP = axis2_line_stride(n2);
    const int k0 = L * blockIdx.x;
    const int kk = threadIdx.x / TL, t = threadIdx.x - kk * TL;
    const int nthr = L * TL;
    const int lsh = L == 4 ? 2 : (L == 2 ? 1 : 0);
#pragma unroll 4
    for (int q = threadIdx.x; q < L * n2; q += nthr) {
        const int y = q >> lsh, j = q & (L - 1);
        if (k0 + j < nc) lines[j * LP + pad16(y)] = spec[(int64_t)y * ncp + k0 + j];
    }
    __syncthreads();
    C* a = lines + kk * LP;
    fft_line<-1, MIX>(a, f, tws, t, TL);
    if (MUL) {
#pragma unroll 4
        for (int q = threadIdx.x; q < L * n2; q += nthr) {
            const int y = q >> lsh, j = q & (L - 1);
            if (k0 + j < nc) lines[j * LP + pad16(y)] = cmul(lines[j * LP + pad16(y)], ks[(int64_t)y * ncp + k0 + j]);
        }
        __syncthreads();
        fft_line<1, MIX>(a, f, tws, t, TL);
    }
    C* dst = MUL ? spec : out;
    for (int q = threadIdx.x; q < L * n2; q += nthr) {
        const int y = q >> lsh, j = q & (L - 1);
        if (k0 + j < nc) dst[(int64_t)y * ncp + k0 + j] = lines[j * LP + pad16(y)];
    }
}

template <typename T>
__device__ __forceinline__ T growth(T u, T U, T mu, T sigma, T dt) {
    const T d = U - mu;
    const T g = T(2) * exp(-(d * d) / (T(2) * (sigma * sigma))) - T(1);
    T v = u + dt * g;
    v = v < T(0) ? T(0) : v;
    return v > T(1) ? T(1) : v;
}

// Step 3: the CTA's lines back along axis 1. Each complex line reads its two lines' rows of half
// spectra, made Hermitian (the imaginary parts of frequencies 0 and n1/2 dropped), as Fa + i Fb
// over all n1 frequencies; its inverse transform holds the two real fields. Then LENIA:
// out = growth(u, U) (pitch pe), and with `next` the new state's lines are transformed at once
// (step 1 of the next step, on the same lines, in the same shared memory) into the same rows of
// spec; else out = U (packed).
template <typename T, bool LENIA, bool MIX>
__global__ void __launch_bounds__(kFftMaxThreads, 1) k_axis1_inverse(typename CxOf<T>::type* __restrict__ spec, int n1, int n2, FftFactors f,
                                const typename CxOf<T>::type* __restrict__ tw, int ntw, const T* __restrict__ u,
                                T* __restrict__ out, int64_t pe, T mu, T sigma, T dt, bool next) {
    using C = typename CxOf<T>::type;
    extern __shared__ __align__(16) unsigned char smem[];
    C* tws = (C*)smem;
    stage_twiddles(tws, tw, ntw);
    const int TL = line_threads(n1);
    const int li = threadIdx.x / TL, t = threadIdx.x - li * TL;
    const int64_t ya = (int64_t)kAxis1Lines * blockIdx.x + 2 * li;
    const bool h0 = ya < n2, h1 = ya + 1 < n2;
    const int ncp = spec_pitch(n1);
    C* a = tws + ntw + li * padded_len(n1);
    {
        const C* ra = spec + ya * ncp;
#pragma unroll 4
        for (int k = t; k < n1; k += TL) {
            const bool lo = 2 * k <= n1;
            const int m = lo ? k : n1 - k;
            C fa = h0 ? ra[m] : C{T(0), T(0)}, fb = h1 ? ra[ncp + m] : C{T(0), T(0)};
            if (!lo) {
                fa.y = -fa.y;
                fb.y = -fb.y;
            }
            if (k == 0 || 2 * k == n1) {
                fa.y = T(0);
                fb.y = T(0);
            }
            a[pad16(k)] = C{fa.x - fb.y, fa.y + fb.x};  // Fa + i Fb
        }
    }
    __syncthreads();
    fft_line<1, MIX>(a, f, tws, t, TL);
    for (int x = t; x < n1; x += TL) {
        const C v = a[pad16(x)];
        if (LENIA) {
            const T g0 = h0 ? growth<T>(u[x + ya * pe], v.x, mu, sigma, dt) : T(0);
            const T g1 = h1 ? growth<T>(u[x + (ya + 1) * pe], v.y, mu, sigma, dt) : T(0);
            if (h0) out[x + ya * pe] = g0;
            if (h1) out[x + (ya + 1) * pe] = g1;
            a[pad16(x)] = C{g0, g1};  // this thread's own slot: the next step's input line
        } else {
            if (h0) out[x + ya * n1] = v.x;
            if (h1) out[x + (ya + 1) * n1] = v.y;
        }
    }
    if (LENIA && next) {  // uniform over the CTA
        __syncthreads();
        fft_line<-1, MIX>(a, f, tws, t, TL);
        split_rows<T>(a, n1, spec + ya * ncp, ncp, h0, h1, t, TL);
    }
}

// ----------------------------------------------- power-of-two lines of compile-time length
// Lines of N = 512, 1024, 2048 or 4096 points (the usual lattice sides) run Stockham stages with
// every index known at compile time but the thread's own. A thread holds P points (P = 8 or 16):
// a first stage of radix P (l = 1, no twiddles), middle stages of radix P (l = P, P^2, ...), and
// a last stage of radix R = N / LL (l = LL). Thread t < N / P holds the first stage's inputs
// x[t + q N / P] and the last stage's outputs X[t + q N / P] (q < P) in registers: the same
// points. So a forward transform's outputs feed the inverse's first stage (the axis-2 product
// between them), an inverse's outputs feed the growth and the next step's forward transform,
// and loads and stores of whole lines go straight between global memory and registers, each
// transform passing through shared memory only between its stages.
constexpr int kPts1 = 8, kPts2 = 16;  // points a thread in the compile-time kernels: axis 1, axis 2

template <int N, int P>
struct PL {
    static_assert(N == 512 || N == 1024 || N == 2048 || N == 4096, "a power-of-two line of 512 .. 4096 points");
    static_assert(P == 8 || P == 16, "8 or 16 points a thread");
    static constexpr int LOG = N == 512 ? 9 : (N == 1024 ? 10 : (N == 2048 ? 11 : 12));
    static constexpr int T = N / P;  // threads a line
    // P = 8: radix 8, 8, ... then 8, 4 or 2 (N = 8^a 2^b); P = 16: radix 16, 16, then N / 256
    static constexpr int RL = P == 8 ? (LOG % 3 == 0 ? 8 : (LOG % 3 == 2 ? 4 : 2)) : N / 256;
    static constexpr int LL = N / RL;      // the last stage's sub-transform length
    static constexpr int TS = T + T / 16;  // slots from point e to e + T
};

// The first stage from registers (v[q] = x[t + q T]) into points P t + m (slots pad16(P t) + m).
template <int P, int DIR, typename C>
__device__ __forceinline__ void pl_first(C* x, C (&v)[P], int t) {
    dft_small<P, DIR>(v);
    C* o = x + pad16(P * t);
#pragma unroll
    for (int m = 0; m < P; ++m) o[m] = v[m];
}

// A middle stage of radix P with sub-transform length L (8 or a multiple of 16), in place:
// butterfly t reads points t + q T, writes points (t - k) P + k + m L (k = t mod L); a barrier
// between the reads and the writes and one after.
template <int N, int P, int DIR, int L, typename C>
__device__ __forceinline__ void pl_middle(C* x, const C* tw, int t) {
    static_assert((L == 8 && P == 8) || L % 16 == 0, "slot offsets below assume L = 8 or a multiple of 16");
    constexpr int TS = PL<N, P>::TS;
    const int k = t & (L - 1);
    const C* in = x + pad16(t);
    const C* w = tw + (L - 1) + k;  // the stage's table follows the earlier stages' L - 1 entries
    C v[P];
    v[0] = in[0];
#pragma unroll
    for (int q = 1; q < P; ++q) {
        C c = w[(q - 1) * L];
        if (DIR > 0) c.y = -c.y;
        v[q] = cmul(in[q * TS], c);
    }
    dft_small<P, DIR>(v);
    __syncthreads();
    C* o = x + pad16((t - k) * P + k);
#pragma unroll
    for (int m = 0; m < P; ++m) o[L == 8 ? 8 * m + (m >> 1) : m * (L + L / 16)] = v[m];
    __syncthreads();
}

template <int N, int P, int DIR, int L, typename C>
__device__ __forceinline__ void pl_middles(C* x, const C* tw, int t) {
    if constexpr (L < PL<N, P>::LL) {
        pl_middle<N, P, DIR, L>(x, tw, t);
        pl_middles<N, P, DIR, L * P>(x, tw, t);
    }
}

// The last stage into registers: v[q] = X[t + q T]. Leaves shared memory being read.
template <int N, int P, int DIR, typename C>
__device__ __forceinline__ void pl_last(const C* x, const C* tw, int t, C (&v)[P]) {
    constexpr int R = PL<N, P>::RL, L = PL<N, P>::LL, B = P / R, T = PL<N, P>::T, TS = PL<N, P>::TS;
    constexpr int LS = L + L / 16;
    const C* in = x + pad16(t);
    const C* w = tw + (L - 1);
#pragma unroll
    for (int b = 0; b < B; ++b) {
        const int j = t + b * T;  // < L: its own k
        C u[R];
        u[0] = in[b * TS];
#pragma unroll
        for (int q = 1; q < R; ++q) {
            C c = w[(q - 1) * L + j];
            if (DIR > 0) c.y = -c.y;
            u[q] = cmul(in[b * TS + q * LS], c);
        }
        dft_small<R, DIR>(u);
#pragma unroll
        for (int m = 0; m < R; ++m) v[b + m * B] = u[m];  // point j + m L = t + (b + m B) T
    }
}

// One line's DFT (exponent sign DIR) from registers to registers through x (the line's padded
// slots, free on entry; still being read on return), in two parts: pl_first, then a barrier and
// the rest (so that a caller can wait for its asynchronous copies in between).
template <int N, int P, int DIR, typename C>
__device__ __forceinline__ void pl_rest(C* x, const C* tw, int t, C (&v)[P]) {
    __syncthreads();
    pl_middles<N, P, DIR, P>(x, tw, t);
    pl_last<N, P, DIR>(x, tw, t, v);
}

// Asynchronous 16-byte copies global -> shared (cp.async, cached in L2 only): the 16-byte chunks
// of `bytes` (a multiple of 16; both addresses 16-byte aligned) by the CTA's threads, then one
// commit group.
__device__ __forceinline__ void copy_async16(void* dst, const void* src, int bytes) {
    const uint32_t d = (uint32_t)__cvta_generic_to_shared(dst);
    for (int i = threadIdx.x; i < bytes / 16; i += blockDim.x)
        asm volatile("cp.async.cg.shared.global [%0], [%1], 16;" ::"r"(d + 16u * i), "l"((const char*)src + 16 * i)
                     : "memory");
    asm volatile("cp.async.commit_group;" ::: "memory");
}
__device__ __forceinline__ void commit_empty() { asm volatile("cp.async.commit_group;" ::: "memory"); }
template <int PENDING>
__device__ __forceinline__ void wait_async() {  // all but the PENDING most recent groups have landed
    asm volatile("cp.async.wait_group %0;" ::"n"(PENDING) : "memory");
}
// A per-stage twiddle table's bytes rounded up to 16 (the tables are allocated one entry long).
__host__ __device__ constexpr int tw_bytes16(int ntw) { return (ntw * 8 + 15) / 16 * 16; }

// Axis-2 lines a CTA: two while that keeps a CTA within 256 threads (two CTAs an SM of up to 128
// registers a thread); thread i takes line i mod L and point index t = i / L, so a warp's loads
// and stores cover 32 / L rows of L consecutive frequencies. Line stride: 8 slots modulo 16 (64
// bytes modulo 128), so that lines kk and kk + 1 fall in different banks. (With 8 points a
// thread, two 256-thread lines a CTA ran a 2048^2 Lenia step in 51.8 us, four in 53.4, one in
// 62.2.)
template <int N, int P> __host__ __device__ constexpr int pl_axis2_lines() { return N / P <= 128 ? 2 : 1; }
template <int N> __host__ __device__ constexpr int pl_axis2_stride() {
    return ((N - 1) + ((N - 1) >> 4) + 1 + 15) / 16 * 16 + 8;  // padded_len(N) rounded up to 16, + 8
}
template <int N, int P> __host__ __device__ constexpr int pl_axis2_smem(int ntw) {  // bytes
    return tw_bytes16(ntw) + 8 * pl_axis2_lines<N, P>() * (N + pl_axis2_stride<N>());
}

// Step 2 for Float32 lines of N points along axis 2: forward transform, product with the
// kernel's spectrum, inverse transform, the L frequencies L blockIdx.x + kk of spec in place.
// The twiddles and the CTA's rows of the kernel's spectrum (L consecutive frequencies, 8 L bytes
// a row) are copied into shared memory asynchronously while the lines load and the forward
// transform runs.
template <int N, int P>
__global__ void __launch_bounds__(pl_axis2_lines<N, P>() * PL<N, P>::T, 2)
    k_pl_axis2(float2* __restrict__ spec, const float2* __restrict__ ks, int n1, const float2* __restrict__ tw,
               int ntw) {
    constexpr int L = pl_axis2_lines<N, P>(), T = PL<N, P>::T;
    extern __shared__ __align__(16) unsigned char smem[];
    float2* tws = (float2*)smem;
    float2* kss = (float2*)(smem + tw_bytes16(ntw));  // row y, frequency col0 + kk at [y L + kk]
    float2* lines = kss + N * L;                       // line kk at lines + kk stride
    const int ncp = spec_pitch(n1), col0 = L * blockIdx.x;
    copy_async16(tws, tw, tw_bytes16(ntw));
    {   // one 8 L-byte piece a row (col0 a multiple of L, ncp of 4: 16-byte aligned for L = 2)
        const uint32_t d = (uint32_t)__cvta_generic_to_shared(kss);
        for (int y = threadIdx.x; y < N; y += blockDim.x) {
            const float2* g = ks + (int64_t)y * ncp + col0;
            if constexpr (L == 2)
                asm volatile("cp.async.cg.shared.global [%0], [%1], 16;" ::"r"(d + 16u * y), "l"(g) : "memory");
            else
                asm volatile("cp.async.ca.shared.global [%0], [%1], 8;" ::"r"(d + 8u * y), "l"(g) : "memory");
        }
        commit_empty();
    }
    const int kk = threadIdx.x % L, t = threadIdx.x / L;
    const int col = col0 + kk;
    const bool ok = col < n1 / 2 + 1;
    float2* x = lines + kk * pl_axis2_stride<N>();
    float2 v[P];
#pragma unroll
    for (int q = 0; q < P; ++q) v[q] = ok ? spec[(int64_t)(t + q * T) * ncp + col] : float2{0.f, 0.f};
    pl_first<P, -1>(x, v, t);
    wait_async<1>();  // the twiddles
    pl_rest<N, P, -1>(x, tws, t, v);
    wait_async<0>();  // the kernel's spectrum
    __syncthreads();  // ... visible to all, and every thread's last-stage reads done
#pragma unroll
    for (int q = 0; q < P; ++q) v[q] = cmul(v[q], kss[(t + q * T) * L + kk]);
    pl_first<P, 1>(x, v, t);
    pl_rest<N, P, 1>(x, tws, t, v);
#pragma unroll
    for (int q = 0; q < P; ++q)
        if (ok) spec[(int64_t)(t + q * T) * ncp + col] = v[q];
}

// The transformed line (registers, natural order) into shared memory, split into the two
// lines' half spectra (rows ya, ya + 1 of spec).
template <int N, int P>
__device__ __forceinline__ void pl_split(float2* a, float2 (&v)[P], float2* ra, int ncp, bool h0, bool h1, int t) {
    constexpr int TS = PL<N, P>::TS;
    __syncthreads();  // the last stage's reads are done
#pragma unroll
    for (int q = 0; q < P; ++q) a[pad16(t) + q * TS] = v[q];
    __syncthreads();
    split_rows<float>(a, N, ra, ncp, h0, h1, t, PL<N, P>::T);
}

// Axis-1 kernels: one complex line (two real lines, N / P threads) a CTA (with 8 points a thread,
// two such lines a CTA ran a 2048^2 Lenia step in 55.9 us against 51.8; twiddles read from
// global memory instead of shared, 59.8).
template <int N> __host__ __device__ constexpr int pl_axis1_line_bytes() {  // the line's slots, to 16 bytes
    return (8 * ((N - 1) + ((N - 1) >> 4) + 1) + 15) / 16 * 16;
}
template <int N> __host__ __device__ constexpr int pl_axis1_smem(int ntw, bool lenia) {  // bytes
    return tw_bytes16(ntw) + pl_axis1_line_bytes<N>() + (lenia ? 2 * 4 * N : 0);
}

// Step 1 for Float32 lines of N points along axis 1: lines 2 b and 2 b + 1 (b = blockIdx.x) as
// one complex line.
template <int N, int P>
__global__ void __launch_bounds__(PL<N, P>::T) k_pl_axis1_forward(const void* __restrict__ u, int64_t pitch, int src,
                                                                  int n2, const float2* __restrict__ tw, int ntw,
                                                                  float2* __restrict__ spec) {
    constexpr int T = PL<N, P>::T;
    extern __shared__ __align__(16) unsigned char smem[];
    float2* tws = (float2*)smem;
    float2* a = (float2*)(smem + tw_bytes16(ntw));
    copy_async16(tws, tw, tw_bytes16(ntw));
    const int t = threadIdx.x;
    const int64_t ya = 2 * (int64_t)blockIdx.x;
    const bool h0 = ya < n2, h1 = ya + 1 < n2;
    float2 v[P];
#pragma unroll
    for (int q = 0; q < P; ++q) {
        const int x = t + q * T;
        v[q] = float2{h0 ? load_source<float>(u, pitch, x, ya, src) : 0.f,
                      h1 ? load_source<float>(u, pitch, x, ya + 1, src) : 0.f};
    }
    pl_first<P, -1>(a, v, t);
    wait_async<0>();  // the twiddles
    pl_rest<N, P, -1>(a, tws, t, v);
    const int ncp = spec_pitch(N);
    pl_split<N, P>(a, v, spec + ya * ncp, ncp, h0, h1, t);
}

// Step 3 for Float32 lines of N points along axis 1, as k_axis1_inverse: the Hermitian halves of
// rows ya, ya + 1 as one complex line straight into the first stage's registers; the inverse's
// outputs to the growth (LENIA; with `next`, on to the next step's forward transform) or to
// the field (packed). The twiddles and, for the growth, the two state lines (pitch pe; rows
// 16-byte aligned) are copied into shared memory asynchronously meanwhile.
template <int N, int P, bool LENIA>
__global__ void __launch_bounds__(PL<N, P>::T) k_pl_axis1_inverse(float2* __restrict__ spec, int n2,
                                                                  const float2* __restrict__ tw, int ntw,
                                                                  const float* __restrict__ u, float* __restrict__ out,
                                                                  int64_t pe, float mu, float sigma, float dt,
                                                                  bool next) {
    constexpr int T = PL<N, P>::T;
    extern __shared__ __align__(16) unsigned char smem[];
    float2* tws = (float2*)smem;
    float2* a = (float2*)(smem + tw_bytes16(ntw));
    float* us = (float*)((unsigned char*)a + pl_axis1_line_bytes<N>());  // state lines ya, ya + 1 (LENIA)
    const int t = threadIdx.x;
    const int64_t ya = 2 * (int64_t)blockIdx.x;
    const bool h0 = ya < n2, h1 = ya + 1 < n2;
    copy_async16(tws, tw, tw_bytes16(ntw));
    if constexpr (LENIA) {
        if (h0) copy_async16(us, u + ya * pe, 4 * N);
        else commit_empty();
        if (h1) copy_async16(us + N, u + (ya + 1) * pe, 4 * N);
        else commit_empty();
    }
    const int ncp = spec_pitch(N);
    const float2* ra = spec + ya * ncp;
    float2 v[P];
#pragma unroll
    for (int q = 0; q < P; ++q) {
        const int k = t + q * T;
        const bool lo = q < P / 2 || (q == P / 2 && t == 0);  // 2 k <= N
        const int m = lo ? k : N - k;
        float2 fa = h0 ? ra[m] : float2{0.f, 0.f}, fb = h1 ? ra[ncp + m] : float2{0.f, 0.f};
        if (!lo) {
            fa.y = -fa.y;
            fb.y = -fb.y;
        }
        if (k == 0 || 2 * k == N) {
            fa.y = 0.f;
            fb.y = 0.f;
        }
        v[q] = float2{fa.x - fb.y, fa.y + fb.x};  // Fa + i Fb
    }
    pl_first<P, 1>(a, v, t);
    if constexpr (LENIA) wait_async<2>();  // the twiddles
    else wait_async<0>();
    pl_rest<N, P, 1>(a, tws, t, v);
    if constexpr (LENIA) {
        wait_async<0>();  // the state lines
        __syncthreads();  // ... visible to all, and every thread's last-stage reads done
#pragma unroll
        for (int q = 0; q < P; ++q) {
            const int x = t + q * T;
            const float g0 = h0 ? growth<float>(us[x], v[q].x, mu, sigma, dt) : 0.f;
            const float g1 = h1 ? growth<float>(us[N + x], v[q].y, mu, sigma, dt) : 0.f;
            if (h0) out[x + ya * pe] = g0;
            if (h1) out[x + (ya + 1) * pe] = g1;
            v[q] = float2{g0, g1};
        }
        if (next) {  // uniform over the CTA
            pl_first<P, -1>(a, v, t);
            pl_rest<N, P, -1>(a, tws, t, v);
            pl_split<N, P>(a, v, spec + ya * ncp, ncp, h0, h1, t);
        }
    } else {
#pragma unroll
        for (int q = 0; q < P; ++q) {
            const int x = t + q * T;
            if (h0) out[x + ya * N] = v[q].x;
            if (h1) out[x + (ya + 1) * N] = v[q].y;
        }
    }
}

// The kernel's spectrum for the per-step product: conj(S) / (n1 n2) in the plan's precision.
template <typename C>
__global__ void k_finish_kspec(const double2* __restrict__ s, C* __restrict__ ks, int64_t n, double scale) {
    for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x) {
        const double2 v = s[i];
        ks[i] = C{(decltype(C{}.x))(v.x * scale), (decltype(C{}.x))(-v.y * scale)};
    }
}

template <typename C>
std::vector<C> radix_table(const std::vector<int>& radices) {
    std::vector<C> t;
    const double pi = 3.14159265358979323846;
    int l = 1;
    for (const int R : radices) {
        for (int q = 1; q < R; ++q)
            for (int k = 0; k < l; ++k) {
                const double a = -2.0 * pi * (double)k * (double)q / (double)(R * l);
                t.push_back(C{(decltype(C{}.x))std::cos(a), (decltype(C{}.x))std::sin(a)});
            }
        l *= R;
    }
    return t;
}

template <typename C>
std::vector<C> stage_table(const FftFactors& f) {
    std::vector<int> r;
    for (int s = 0; s < f.nst; ++s) r.push_back(f.radix(s));
    return radix_table<C>(r);
}

}  // namespace

struct SpecConv {
    int64_t n1 = 0, n2 = 0;
    bool f64 = false;
    FftFactors f1{}, f2{};
    int ntw1 = 0, ntw2 = 0;  // entries of the per-stage twiddle tables
    void* tw1 = nullptr;  // twiddles of axis 1 and 2 in the plan's precision
    void* tw2 = nullptr;
    void* tw16[2] = {nullptr, nullptr};  // Float32 tables of the 16-point plans (radix 16, 16, n / 256), axes 1, 2
    void* ks = nullptr;    // conj(rfft2(kpad)) / (n1 n2), frequency-major: [k][ky]
    void* spec = nullptr;  // work spectrum, the same layout
};

bool specconv_supported(int64_t n1, int64_t n2, bool f64) {
    // a CTA transforms two axis-1 lines (2 x line_threads(n1) <= 1024 threads) or up to four
    // axis-2 lines (line_threads(n2) <= 1024); shared memory holds them and their twiddles
    if (n1 < 1 || n2 < 1 || n1 > 4096 || n2 > 8192) return false;
    const FftFactors f1 = factorize(n1), f2 = factorize(n2);
    if (f1.nst < 0 || f2.nst < 0) return false;
    const size_t cs = f64 ? sizeof(double2) : sizeof(float2);
    const size_t s1 = cs * (size_t)(twiddle_count(f1) + 2 * padded_len((int)n1));
    const size_t s2 = cs * (size_t)(twiddle_count(f2) + axis2_lines((int)n2) * axis2_line_stride((int)n2));
    return s1 <= (size_t)smem_optin() && s2 <= (size_t)smem_optin();
}

void specconv_destroy(SpecConv* p) {
    if (!p) return;
    cudaFree(p->tw1);
    cudaFree(p->tw2);
    cudaFree(p->tw16[0]);
    cudaFree(p->tw16[1]);
    cudaFree(p->ks);
    cudaFree(p->spec);
    delete p;
}

namespace {

bool pow2(int64_t n) { return n > 0 && (n & (n - 1)) == 0; }

template <typename T, bool MIX>
cudaError_t launch_axis1_forward(SpecConv* p, const void* u, int64_t pitch, int src, const void* tw, void* spec,
                                 cudaStream_t st) {
    using C = typename CxOf<T>::type;
    const int n1 = (int)p->n1, n2 = (int)p->n2;
    const size_t smem = sizeof(C) * (size_t)(p->ntw1 + kAxis1Complex * padded_len(n1));
    cudaError_t e = ensure_dynamic_smem((const void*)k_axis1_forward<T, MIX>, smem);
    if (e != cudaSuccess) return e;
    const unsigned grid = (unsigned)((n2 + kAxis1Lines - 1) / kAxis1Lines);
    k_axis1_forward<T, MIX><<<grid, kAxis1Complex * line_threads(n1), smem, st>>>(u, pitch, src, n1, n2, p->f1, (const C*)tw,
                                                                       p->ntw1, (C*)spec);
    count_launch();
    return cudaGetLastError();
}

template <typename T, bool MUL, bool MIX>
cudaError_t launch_axis2(SpecConv* p, void* spec, const void* ks, void* out, const void* tw, cudaStream_t st) {
    using C = typename CxOf<T>::type;
    const int n1 = (int)p->n1, n2 = (int)p->n2, L = axis2_lines(n2);
    const size_t smem = sizeof(C) * (size_t)(p->ntw2 + L * axis2_line_stride(n2));
    cudaError_t e = ensure_dynamic_smem((const void*)k_axis2<T, MUL, MIX>, smem);
    if (e != cudaSuccess) return e;
    const unsigned grid = (unsigned)((n1 / 2 + 1 + L - 1) / L);
    k_axis2<T, MUL, MIX><<<grid, L * line_threads(n2), smem, st>>>((C*)spec, (const C*)ks, (C*)out, n1, n2, p->f2,
                                                                   (const C*)tw, p->ntw2);
    count_launch();
    return cudaGetLastError();
}

template <typename T, bool LENIA, bool MIX>
cudaError_t launch_axis1_inverse(SpecConv* p, const T* u, T* out, int64_t pe, double mu, double sigma, double dt,
                                 bool next, cudaStream_t st) {
    using C = typename CxOf<T>::type;
    const int n1 = (int)p->n1, n2 = (int)p->n2;
    const size_t smem = sizeof(C) * (size_t)(p->ntw1 + kAxis1Complex * padded_len(n1));
    cudaError_t e = ensure_dynamic_smem((const void*)k_axis1_inverse<T, LENIA, MIX>, smem);
    if (e != cudaSuccess) return e;
    const unsigned grid = (unsigned)((n2 + kAxis1Lines - 1) / kAxis1Lines);
    k_axis1_inverse<T, LENIA, MIX><<<grid, kAxis1Complex * line_threads(n1), smem, st>>>(
        (C*)p->spec, n1, n2, p->f1, (const C*)p->tw1, p->ntw1, u, out, pe, (T)mu, (T)sigma, (T)dt, next);
    count_launch();
    return cudaGetLastError();
}

// Points a thread in the compile-time kernels: 8 on axis 1, 16 on axis 2 (2048^2 Lenia step:
// 45.3 us; 8 and 8: 47.4; 16 and 16: 47.1; 16 and 8: 49.5).
// A compile-time kernel's twiddle table: the 8-point plan's is the general plan's (radix 8, ...,
// then 4 or 2); the 16-point plan (radix 16, 16, n / 256) has its own.
inline const float2* pl_table(const SpecConv* p, int axis, int pts) {
    return (const float2*)(pts == 16 ? p->tw16[axis] : (axis == 0 ? p->tw1 : p->tw2));
}

template <int N>
cudaError_t pl_axis1_forward(SpecConv* p, const void* u, int64_t pitch, int src, void* spec, cudaStream_t st) {
    constexpr int P = kPts1;
    const size_t smem = (size_t)pl_axis1_smem<N>(N - 1, false);
    cudaError_t e = ensure_dynamic_smem((const void*)k_pl_axis1_forward<N, P>, smem);
    if (e != cudaSuccess) return e;
    k_pl_axis1_forward<N, P><<<(unsigned)((p->n2 + 1) / 2), PL<N, P>::T, smem, st>>>(
        u, pitch, src, (int)p->n2, pl_table(p, 0, P), N - 1, (float2*)spec);
    count_launch();
    return cudaGetLastError();
}

template <int N>
cudaError_t pl_axis2(SpecConv* p, cudaStream_t st) {
    constexpr int P = kPts2, L = pl_axis2_lines<N, P>();
    const size_t smem = (size_t)pl_axis2_smem<N, P>(N - 1);
    cudaError_t e = ensure_dynamic_smem((const void*)k_pl_axis2<N, P>, smem);
    if (e != cudaSuccess) return e;
    k_pl_axis2<N, P><<<(unsigned)((p->n1 / 2 + 1 + L - 1) / L), L * PL<N, P>::T, smem, st>>>(
        (float2*)p->spec, (const float2*)p->ks, (int)p->n1, pl_table(p, 1, P), N - 1);
    count_launch();
    return cudaGetLastError();
}

template <int N, bool LENIA>
cudaError_t pl_axis1_inverse(SpecConv* p, const float* u, float* out, int64_t pe, double mu, double sigma, double dt,
                             bool next, cudaStream_t st) {
    constexpr int P = kPts1;
    const size_t smem = (size_t)pl_axis1_smem<N>(N - 1, LENIA);
    cudaError_t e = ensure_dynamic_smem((const void*)k_pl_axis1_inverse<N, P, LENIA>, smem);
    if (e != cudaSuccess) return e;
    k_pl_axis1_inverse<N, P, LENIA><<<(unsigned)((p->n2 + 1) / 2), PL<N, P>::T, smem, st>>>(
        (float2*)p->spec, (int)p->n2, pl_table(p, 0, P), N - 1, u, out, pe, (float)mu, (float)sigma, (float)dt,
        next);
    count_launch();
    return cudaGetLastError();
}

// Step 1 alone: the lines of u along axis 1 into spec.
template <typename T>
cudaError_t run_axis1(SpecConv* p, const void* u, int64_t pitch, int src, const void* tw1, void* spec, cudaStream_t st) {
    if constexpr (std::is_same<T, float>::value) {
        switch (p->n1) {
            case 512: return pl_axis1_forward<512>(p, u, pitch, src, spec, st);
            case 1024: return pl_axis1_forward<1024>(p, u, pitch, src, spec, st);
            case 2048: return pl_axis1_forward<2048>(p, u, pitch, src, spec, st);
            case 4096: return pl_axis1_forward<4096>(p, u, pitch, src, spec, st);
            default: break;
        }
    }
    return pow2(p->n1) ? launch_axis1_forward<T, false>(p, u, pitch, src, tw1, spec, st)
                       : launch_axis1_forward<T, true>(p, u, pitch, src, tw1, spec, st);
}

// Step 2: with mul, the spectral product and the inverse along axis 2 in spec; without, the
// forward spectrum into out.
template <typename T>
cudaError_t run_axis2(SpecConv* p, void* spec, const void* ks, void* out, const void* tw2, bool mul, cudaStream_t st) {
    if constexpr (std::is_same<T, float>::value) {
        if (mul && spec == p->spec && ks == p->ks && tw2 == p->tw2) switch (p->n2) {
                case 512: return pl_axis2<512>(p, st);
                case 1024: return pl_axis2<1024>(p, st);
                case 2048: return pl_axis2<2048>(p, st);
                case 4096: return pl_axis2<4096>(p, st);
                default: break;
            }
    }
    const bool m2 = !pow2(p->n2);
    if (mul) return m2 ? launch_axis2<T, true, true>(p, spec, ks, nullptr, tw2, st)
                       : launch_axis2<T, true, false>(p, spec, ks, nullptr, tw2, st);
    return m2 ? launch_axis2<T, false, true>(p, spec, nullptr, out, tw2, st)
              : launch_axis2<T, false, false>(p, spec, nullptr, out, tw2, st);
}

// Step 3: Lenia's growth into out (pitch pe; with next, the new state's step 1 too), or the
// field into out (packed).
template <typename T>
cudaError_t run_inverse(SpecConv* p, const T* u, T* out, int64_t pe, bool lenia, double mu, double sigma, double dt,
                        bool next, cudaStream_t st) {
    if constexpr (std::is_same<T, float>::value) {
        switch (p->n1) {
            case 512: return lenia ? pl_axis1_inverse<512, true>(p, u, out, pe, mu, sigma, dt, next, st)
                                   : pl_axis1_inverse<512, false>(p, u, out, pe, mu, sigma, dt, false, st);
            case 1024: return lenia ? pl_axis1_inverse<1024, true>(p, u, out, pe, mu, sigma, dt, next, st)
                                    : pl_axis1_inverse<1024, false>(p, u, out, pe, mu, sigma, dt, false, st);
            case 2048: return lenia ? pl_axis1_inverse<2048, true>(p, u, out, pe, mu, sigma, dt, next, st)
                                    : pl_axis1_inverse<2048, false>(p, u, out, pe, mu, sigma, dt, false, st);
            case 4096: return lenia ? pl_axis1_inverse<4096, true>(p, u, out, pe, mu, sigma, dt, next, st)
                                    : pl_axis1_inverse<4096, false>(p, u, out, pe, mu, sigma, dt, false, st);
            default: break;
        }
    }
    const bool m1 = !pow2(p->n1);
    if (lenia)
        return m1 ? launch_axis1_inverse<T, true, true>(p, u, out, pe, mu, sigma, dt, next, st)
                  : launch_axis1_inverse<T, true, false>(p, u, out, pe, mu, sigma, dt, next, st);
    return m1 ? launch_axis1_inverse<T, false, true>(p, u, out, pe, mu, sigma, dt, false, st)
              : launch_axis1_inverse<T, false, false>(p, u, out, pe, mu, sigma, dt, false, st);
}

// nsteps Lenia steps: step 1 of the first, then per step the axis-2 product and the inverse
// with the growth, which also runs step 1 of the following step (all but the last).
template <typename T>
cudaError_t lenia_run(SpecConv* p, void* const bufs[2], int* cur, int64_t nsteps, int64_t pe, double mu,
                      double sigma, double dt, cudaStream_t st) {
    if (nsteps <= 0) return cudaSuccess;
    cudaError_t e = run_axis1<T>(p, bufs[*cur], pe, kSpecReal, p->tw1, p->spec, st);
    for (int64_t s = 0; s < nsteps && e == cudaSuccess; ++s) {
        e = run_axis2<T>(p, p->spec, p->ks, nullptr, p->tw2, true, st);
        if (e == cudaSuccess)
            e = run_inverse<T>(p, (const T*)bufs[*cur], (T*)bufs[*cur ^ 1], pe, true, mu, sigma, dt, s + 1 < nsteps,
                               st);
        if (e == cudaSuccess) *cur ^= 1;
    }
    return e;
}

}  // namespace

int specconv_create(int64_t n1, int64_t n2, bool f64, const double* kpad, cudaStream_t st, SpecConv** out,
                    std::string& err) {
    *out = nullptr;
    if (!specconv_supported(n1, n2, f64)) {
        err = "the lattice's sides are not products of 2, 3 and 5 that fit the transform";
        return GBCA_ERR_UNSUPPORTED;
    }
    SpecConv* p = new SpecConv();
    p->n1 = n1;
    p->n2 = n2;
    p->f64 = f64;
    p->f1 = factorize(n1);
    p->f2 = factorize(n2);
    const int64_t nc = spec_pitch((int)n1), ncell = n1 * n2;  // nc: the spectra's row pitch
    const size_t cs = f64 ? sizeof(double2) : sizeof(float2);
    // FP64 twiddles for the kernel's spectrum; the plan's own in its precision
    p->ntw1 = twiddle_count(p->f1);
    p->ntw2 = twiddle_count(p->f2);
    const std::vector<double2> t1d = stage_table<double2>(p->f1), t2d = stage_table<double2>(p->f2);
    double2 *d_t1 = nullptr, *d_t2 = nullptr, *d_s = nullptr, *d_o = nullptr;
    double* d_k = nullptr;
    cudaError_t e = cudaMalloc(&p->ks, cs * (size_t)(nc * n2));
    if (e == cudaSuccess) e = cudaMalloc(&p->spec, cs * (size_t)(nc * n2));
    if (e == cudaSuccess) e = cudaMalloc(&p->tw1, cs * (size_t)(p->ntw1 + 1));
    if (e == cudaSuccess) e = cudaMalloc(&p->tw2, cs * (size_t)(p->ntw2 + 1));
    if (e == cudaSuccess) e = cudaMalloc(&d_t1, sizeof(double2) * (size_t)(p->ntw1 + 1));
    if (e == cudaSuccess) e = cudaMalloc(&d_t2, sizeof(double2) * (size_t)(p->ntw2 + 1));
    if (e == cudaSuccess) e = cudaMalloc(&d_s, sizeof(double2) * (size_t)(nc * n2));
    if (e == cudaSuccess) e = cudaMalloc(&d_o, sizeof(double2) * (size_t)(nc * n2));
    if (e == cudaSuccess) e = cudaMalloc(&d_k, sizeof(double) * (size_t)ncell);
    if (e == cudaSuccess) e = cudaMemcpyAsync(d_t1, t1d.data(), sizeof(double2) * p->ntw1, cudaMemcpyHostToDevice, st);
    if (e == cudaSuccess) e = cudaMemcpyAsync(d_t2, t2d.data(), sizeof(double2) * p->ntw2, cudaMemcpyHostToDevice, st);
    if (e == cudaSuccess) e = cudaMemcpyAsync(d_k, kpad, sizeof(double) * ncell, cudaMemcpyHostToDevice, st);
    std::vector<float2> t1f, t2f;
    if (e == cudaSuccess) {
        if (f64) {
            e = cudaMemcpyAsync(p->tw1, t1d.data(), sizeof(double2) * p->ntw1, cudaMemcpyHostToDevice, st);
            if (e == cudaSuccess)
                e = cudaMemcpyAsync(p->tw2, t2d.data(), sizeof(double2) * p->ntw2, cudaMemcpyHostToDevice, st);
        } else {
            t1f = stage_table<float2>(p->f1);
            t2f = stage_table<float2>(p->f2);
            e = cudaMemcpyAsync(p->tw1, t1f.data(), sizeof(float2) * p->ntw1, cudaMemcpyHostToDevice, st);
            if (e == cudaSuccess)
                e = cudaMemcpyAsync(p->tw2, t2f.data(), sizeof(float2) * p->ntw2, cudaMemcpyHostToDevice, st);
        }
    }
    std::vector<float2> t16[2];
    for (int a = 0; a < 2 && e == cudaSuccess && !f64; ++a) {
        const int64_t n = a == 0 ? n1 : n2;
        if ((a == 0 ? kPts1 : kPts2) != 16 || (n != 512 && n != 1024 && n != 2048 && n != 4096)) continue;
        t16[a] = radix_table<float2>({16, 16, (int)(n / 256)});
        e = cudaMalloc(&p->tw16[a], sizeof(float2) * (size_t)n);
        if (e == cudaSuccess)
            e = cudaMemcpyAsync(p->tw16[a], t16[a].data(), sizeof(float2) * t16[a].size(), cudaMemcpyHostToDevice, st);
    }
    if (e == cudaSuccess) e = run_axis1<double>(p, d_k, n1, kSpecReal, d_t1, d_s, st);
    if (e == cudaSuccess) e = run_axis2<double>(p, d_s, nullptr, d_o, d_t2, false, st);
    if (e == cudaSuccess) {
        const double scale = 1.0 / (double)ncell;
        if (f64) k_finish_kspec<double2><<<256, 256, 0, st>>>(d_o, (double2*)p->ks, nc * n2, scale);
        else k_finish_kspec<float2><<<256, 256, 0, st>>>(d_o, (float2*)p->ks, nc * n2, scale);
        count_launch();
        e = cudaGetLastError();
    }
    if (e == cudaSuccess) e = cudaStreamSynchronize(st);  // the host vectors and temporaries go out of scope
    cudaFree(d_t1);
    cudaFree(d_t2);
    cudaFree(d_s);
    cudaFree(d_o);
    cudaFree(d_k);
    if (e != cudaSuccess) {
        err = cudaGetErrorString(e);
        const bool oom = e == cudaErrorMemoryAllocation;
        specconv_destroy(p);
        cudaGetLastError();
        return oom ? GBCA_ERR_OUT_OF_MEMORY : GBCA_ERR_CUDA;
    }
    *out = p;
    return GBCA_OK;
}

cudaError_t specconv_lenia_run(SpecConv* p, void* const bufs[2], int* cur, int64_t nsteps, int64_t pe, double mu,
                               double sigma, double dt, cudaStream_t st) {
    return p->f64 ? lenia_run<double>(p, bufs, cur, nsteps, pe, mu, sigma, dt, st)
                  : lenia_run<float>(p, bufs, cur, nsteps, pe, mu, sigma, dt, st);
}

cudaError_t specconv_field(SpecConv* p, const int8_t* u, int64_t pitch, SpecSource src, void* field,
                           cudaStream_t st) {
    cudaError_t e;
    if (p->f64) {
        e = run_axis1<double>(p, u, pitch, src, p->tw1, p->spec, st);
        if (e == cudaSuccess) e = run_axis2<double>(p, p->spec, p->ks, nullptr, p->tw2, true, st);
        if (e == cudaSuccess) e = run_inverse<double>(p, nullptr, (double*)field, 0, false, 0, 0, 0, false, st);
    } else {
        e = run_axis1<float>(p, u, pitch, src, p->tw1, p->spec, st);
        if (e == cudaSuccess) e = run_axis2<float>(p, p->spec, p->ks, nullptr, p->tw2, true, st);
        if (e == cudaSuccess) e = run_inverse<float>(p, nullptr, (float*)field, 0, false, 0, 0, 0, false, st);
    }
    return e;
}

}  // namespace gbca
