// lenia.cu — Lenia (src/lenia.jl:17-47) on the device, in the precision of its state.
//
// The potential U is the kernel field of src/environment.jl:151-169 with the LeniaKernel
// weights of src/kernels.jl:87-104, listed and normalised in FP64 on the host exactly as
// kernel_weights does (src/kernels.jl:174-189) and then cast to the state's precision
// (src/environment.jl:63). Each step is
//     u' = clamp(u + dt * (2 exp(-(U - mu)^2 / (2 sigma^2)) - 1), 0, 1).
//
// Direct field: a fused kernel per step. A CTA stages a tile of u plus a halo of R
// cells in shared memory (periodic / reflecting / Constant(0) through the boundary map);
// each thread computes 16 consecutive cells of a row, sliding a 16+2R register window
// over the kernel rows, so each shared-memory value feeds up to 16 fused multiply-adds.
// R = 13 (the standard Lenia radius) is specialised: the rows dj and -dj (equal weights) summed
// before the multiply-adds, the taps of a row unrolled at compile time, rows of equal extent
// sharing one loop body (a quarter of the code of a fully unrolled disk), the weights in the
// parameter bank, and the kernel persistent: each CTA stages its next tile by cp.async into a
// second buffer while it computes the current one; other radii loop over a tap list.
//
// FFT field (periodic lattices, the FFTW extension's convention
// ext/CellularAutomataCoreFFTWExt.jl:17-30): U = irfft(rfft(u) .* conj(rfft(kpad))) with
// kpad the kernel wrapped onto the lattice. Sides that are products of 2, 3 and 5 run this
// library's own transforms with the growth fused into the last one (spectral.cu: two launches a
// step in a run of steps); other sides run cuFFT (a library call) with this file's spectral product and growth.
#include <cmath>
#include <cstring>
#include <vector>

#include <cufft.h>

#include "gbca_internal.cuh"
#include "lenia.cuh"
#include "spectral.cuh"

namespace gbca {

namespace {

constexpr int kR13 = 13;
constexpr int kBox13 = 2 * kR13 + 1;
constexpr int kDirTX = 128, kDirTY = 32, kDirCells = 16;  // tile and cells per thread

template <typename T>
struct Box13 {
    T w[kBox13 * kBox13];  // dense weights by (dj + R) * 27 + (di + R), offsets already negated
};

constexpr bool in_disk13(int di, int dj) { return di * di + dj * dj < kR13 * kR13 && (di != 0 || dj != 0); }

template <typename T>
__device__ __forceinline__ T growth_step(T u, T U, T mu, T sigma, T dt) {
    const T d = U - mu;
    const T g = T(2) * exp(-(d * d) / (T(2) * (sigma * sigma))) - T(1);
    T v = u + dt * g;
    v = v < T(0) ? T(0) : v;
    return v > T(1) ? T(1) : v;
}

// Tile loader for the direct kernels: lattice values through the boundary map
// (Constant edges of a Lenia problem are Constant(0)).
template <typename T>
__device__ __forceinline__ void load_tile(const T* __restrict__ u, int64_t n1, int64_t n2, int64_t pe, int b1, int b2,
                                          int64_t x0, int64_t y0, int sx, int sy, int sp, T* s) {
    for (int q = threadIdx.x; q < sx * sy; q += blockDim.x) {
        const int lx = q % sx, ly = q / sx;
        const int64_t mx = map_axis(b1, x0 + lx, n1), my = map_axis(b2, y0 + ly, n2);
        s[ly * sp + lx] = (mx < 0 || my < 0) ? T(0) : u[mx + my * pe];
    }
}

// 16 bytes of a 16-byte-aligned shared-memory row into consecutive registers.
template <typename T>
__device__ __forceinline__ void load16(const T* p, T* dst) {
    if constexpr (sizeof(T) == 4) {
        const float4 v = *(const float4*)p;
        dst[0] = v.x;
        dst[1] = v.y;
        dst[2] = v.z;
        dst[3] = v.w;
    } else {
        const double2 v = *(const double2*)p;
        dst[0] = v.x;
        dst[1] = v.y;
    }
}

// Shared row pitch of k_lenia13's tile, in elements: room for the last thread's 16-byte-aligned
// window (cells lx0 - R .. lx0 + 15 + R rounded up to whole 16-byte loads), and a row length of
// 16 bytes modulo 128, so that eight consecutive rows start in eight different groups of four
// banks and a quarter-warp's eight 16-byte loads (one per row) meet no bank conflict.
template <typename T>
constexpr int lenia13_pitch() {
    constexpr int V = 16 / (int)sizeof(T);
    constexpr int need = kDirTX - kDirCells + (kDirCells + 2 * kR13 + V - 1) / V * V;
    int sp = need;
    while ((sp * (int)sizeof(T)) % 128 != 16) ++sp;
    return sp;
}

// Rows dj = D0..D1 of the R = 13 disk (and -dj), whose taps all have |di| <= EXT (di != 0 when
// dj = 0), into the thread's 16 accumulators: the two rows' 16-byte window loads, their sum, then
// one multiply-add per tap and cell, the weight read from the parameter bank by dj. A loop over
// dj (not unrolled) when D1 > D0, so rows of one extent share their code.
template <typename T, int EXT, int D0, int D1>
__device__ __forceinline__ void lenia13_rows(const T* centre, int sp, const Box13<T>& wb, T* acc) {
    constexpr int V = 16 / sizeof(T);
    constexpr int W = kDirCells + 2 * kR13;
    constexpr int WL = (W + V - 1) / V * V;
#pragma unroll 1
    for (int dj = D0; dj <= D1; ++dj) {
        T win[WL];
        if (D0 == 0) {
#pragma unroll
            for (int k = 0; k < WL; k += V) load16<T>(centre + k, win + k);
        } else {
            T lo[WL];
#pragma unroll
            for (int k = 0; k < WL; k += V) {
                load16<T>(centre + dj * sp + k, win + k);
                load16<T>(centre - dj * sp + k, lo + k);
            }
#pragma unroll
            for (int k = 0; k < W; ++k) win[k] += lo[k];
        }
        const T* wrow = wb.w + (dj + kR13) * kBox13 + kR13;
#pragma unroll
        for (int di = -EXT; di <= EXT; ++di) {
            if (D0 == 0 && di == 0) continue;
            const T w = wrow[di];
#pragma unroll
            for (int k = 0; k < kDirCells; ++k) acc[k] = fma(w, win[k + di + kR13], acc[k]);
        }
    }
}

// R = 13. The Lenia kernel depends on the distance only, so rows dj and -dj carry the same
// weights: each thread adds the two rows' windows first (one add per window cell) and then
// runs one fused multiply-add per tap of the pair for each of its 16 cells, 271 per cell for
// the 516 taps (lenia13_rows, by groups of rows of one extent). Windows arrive by 16-byte
// shared-memory loads. Thread layout: the eight lanes of a quarter-warp take eight consecutive
// output rows at the same 16 columns (lanes 8q..8q+7, column block 4 (warp / 4) + q), so with
// lenia13_pitch each of their loads is conflict-free. The tile (X0, Y0) is staged in s.
template <typename T>
__device__ __forceinline__ void lenia13_tile(const T* s, T* __restrict__ out, int64_t n1, int64_t n2, int64_t pe,
                                             int64_t X0, int64_t Y0, const Box13<T>& wb, T mu, T sigma, T dt) {
    constexpr int sp = lenia13_pitch<T>();
    static_assert(kDirTX / kDirCells == 8 && kDirTY == 32, "thread layout: 8 column blocks x 32 rows");
    const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
    const int tx = 4 * (warp >> 2) + (lane >> 3), ty = 8 * (warp & 3) + (lane & 7);
    const int lx0 = tx * kDirCells;                // local x of the first output (tile coords)
    const T* centre = s + (ty + kR13) * sp + lx0;  // the thread's row, from cell lx0 - R
    T acc[kDirCells];
#pragma unroll
    for (int k = 0; k < kDirCells; ++k) acc[k] = T(0);
    // rows with the same tap extent |di| <= EXT share one loop body: dj = 1..4 (12), 5..6 (11),
    // 7..8 (10); the weights of the pair come from the parameter bank by dj
    lenia13_rows<T, 12, 0, 0>(centre, sp, wb, acc);
    lenia13_rows<T, 12, 1, 4>(centre, sp, wb, acc);
    lenia13_rows<T, 11, 5, 6>(centre, sp, wb, acc);
    lenia13_rows<T, 10, 7, 8>(centre, sp, wb, acc);
    lenia13_rows<T, 9, 9, 9>(centre, sp, wb, acc);
    lenia13_rows<T, 8, 10, 10>(centre, sp, wb, acc);
    lenia13_rows<T, 6, 11, 11>(centre, sp, wb, acc);
    lenia13_rows<T, 4, 12, 12>(centre, sp, wb, acc);
    const int64_t gy = Y0 + ty;
    if (gy >= n2) return;
#pragma unroll
    for (int k = 0; k < kDirCells; ++k) {
        const int64_t gx = X0 + lx0 + k;
        if (gx < n1) out[gx + gy * pe] = growth_step<T>(centre[k + kR13], acc[k], mu, sigma, dt);
    }
}

// cp.async of one lattice value into shared memory, or zeros (a source size of 0) beyond a
// Constant(0) edge.
template <typename T>
__device__ __forceinline__ void cp_async_value(T* dst, const T* src, bool zero) {
    const uint32_t d = (uint32_t)__cvta_generic_to_shared(dst);
    asm volatile("cp.async.ca.shared.global [%0], [%1], %2, %3;" ::"r"(d), "l"(src), "n"((int)sizeof(T)),
                 "r"(zero ? 0 : (int)sizeof(T))
                 : "memory");
}

// The halo-padded tile at lattice (x0, y0) into s by asynchronous copies through the boundary
// map, committed as one group.
template <typename T>
__device__ __forceinline__ void stage_tile_async(const T* __restrict__ u, int64_t n1, int64_t n2, int64_t pe, int b1,
                                                 int b2, int64_t x0, int64_t y0, T* s) {
    constexpr int sx = kDirTX + 2 * kR13, sy = kDirTY + 2 * kR13;
    constexpr int sp = lenia13_pitch<T>();
    for (int q = threadIdx.x; q < sx * sy; q += blockDim.x) {
        const int lx = q % sx, ly = q / sx;
        const int64_t mx = map_axis(b1, x0 + lx, n1), my = map_axis(b2, y0 + ly, n2);
        const bool zero = mx < 0 || my < 0;
        cp_async_value<T>(s + ly * sp + lx, zero ? u : u + mx + my * pe, zero);
    }
    asm volatile("cp.async.commit_group;" ::: "memory");
}

// Persistent form: CTA b takes tiles b, b + gridDim.x, ... and stages each next tile into the
// other of two buffers by cp.async while it computes the current one.
template <typename T>
__global__ void __launch_bounds__(256) k_lenia13p(const T* __restrict__ u, T* __restrict__ out, int64_t n1, int64_t n2,
                                                  int64_t pe, int b1, int b2, Box13<T> wb, T mu, T sigma, T dt,
                                                  int tiles_x, int ntiles) {
    extern __shared__ __align__(16) unsigned char lsm[];
    constexpr int sy = kDirTY + 2 * kR13;
    constexpr int sp = lenia13_pitch<T>();
    T* buf0 = (T*)lsm;
    T* buf1 = buf0 + sp * sy;
    int tile = blockIdx.x;
    if (tile < ntiles)
        stage_tile_async<T>(u, n1, n2, pe, b1, b2, (int64_t)(tile % tiles_x) * kDirTX - kR13,
                            (int64_t)(tile / tiles_x) * kDirTY - kR13, buf0);
    for (int i = 0; tile < ntiles; ++i) {
        const int next = tile + (int)gridDim.x;
        T* cur = (i & 1) ? buf1 : buf0;
        if (next < ntiles)
            stage_tile_async<T>(u, n1, n2, pe, b1, b2, (int64_t)(next % tiles_x) * kDirTX - kR13,
                                (int64_t)(next / tiles_x) * kDirTY - kR13, (i & 1) ? buf0 : buf1);
        else
            asm volatile("cp.async.commit_group;" ::: "memory");  // an empty group: the wait below stays one behind
        asm volatile("cp.async.wait_group 1;" ::: "memory");       // this tile's copies have landed
        __syncthreads();
        lenia13_tile<T>(cur, out, n1, n2, pe, (int64_t)(tile % tiles_x) * kDirTX, (int64_t)(tile / tiles_x) * kDirTY,
                        wb, mu, sigma, dt);
        __syncthreads();  // every thread is done with cur before the next iteration refills it
        tile = next;
    }
    asm volatile("cp.async.wait_group 0;" ::: "memory");
}

// Any radius: one cell per thread, taps from a list in global memory (read-only cache).
template <typename T>
__global__ void __launch_bounds__(256) k_lenia_taps(const T* __restrict__ u, T* __restrict__ out, int64_t n1,
                                                    int64_t n2, int64_t pe, int b1, int b2,
                                                    const int2* __restrict__ off, const T* __restrict__ w, int ntaps,
                                                    int R, T mu, T sigma, T dt) {
    extern __shared__ __align__(16) unsigned char lsm[];
    T* s = (T*)lsm;
    const int tile = 32, sx = tile + 2 * R, sy = tile + 2 * R, sp = sx;
    const int64_t X0 = (int64_t)blockIdx.x * tile, Y0 = (int64_t)blockIdx.y * tile;
    load_tile<T>(u, n1, n2, pe, b1, b2, X0 - R, Y0 - R, sx, sy, sp, s);
    __syncthreads();
    for (int q = threadIdx.x; q < tile * tile; q += blockDim.x) {
        const int lx = q % tile, ly = q / tile;
        const int64_t gx = X0 + lx, gy = Y0 + ly;
        if (gx >= n1 || gy >= n2) continue;
        T acc = T(0);
        for (int k = 0; k < ntaps; ++k) {
            const int2 o = __ldg(&off[k]);
            acc = fma(__ldg(&w[k]), s[(ly + R + o.y) * sp + lx + R + o.x], acc);
        }
        out[gx + gy * pe] = growth_step<T>(s[(ly + R) * sp + lx + R], acc, mu, sigma, dt);
    }
}

template <typename C>
__global__ void k_spectral_mul(C* __restrict__ a, const C* __restrict__ k, int64_t n) {
    for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x) {
        const C x = a[i], y = k[i];
        a[i] = C{x.x * y.x - x.y * y.y, x.x * y.y + x.y * y.x};
    }
}

template <typename T>
__global__ void k_growth(const T* __restrict__ u, const T* __restrict__ field, T* __restrict__ out, int64_t n1,
                         int64_t n2, int64_t pe, int64_t fe, T mu, T sigma, T dt) {
    const int64_t n = n1 * n2;
    for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x) {
        const int64_t x = i % n1, y = i / n1;
        out[x + y * pe] = growth_step<T>(u[x + y * pe], field[x + y * fe], mu, sigma, dt);
    }
}

// kernels.jl:96-104
double lenia_value(double d, int R, const double* peaks, int B) {
    const double r = d / (double)R;
    if (r <= 0.0 || r >= 1.0) return 0.0;
    const double x = (double)B * r;
    int64_t i = (int64_t)std::floor(x);
    if (i > B - 1) i = B - 1;
    const double f = x - (double)i;
    return (0.0 < f && f < 1.0) ? peaks[i] * std::exp(4.0 - 1.0 / (f * (1.0 - f))) : 0.0;
}

}  // namespace

namespace {

int fail_to(std::string& err, int code, const char* msg) {
    err = msg;
    return code;
}

}  // namespace

struct LeniaPlan {
    gbca_desc d;
    int64_t n1 = 0, n2 = 0, pe = 0;  // pitch in elements
    bool f64 = false, fft = false, box13 = false;
    std::vector<int> off;            // (di, dj) pairs, negated kernel offsets in kernel_weights order
    std::vector<double> w;           // FP64-normalised weights
    Box13<float> b32;
    Box13<double> b64;
    int2* d_off = nullptr;
    void* d_w = nullptr;
    cufftHandle fwd = 0, inv = 0;
    void* kspec = nullptr;  // conj(rfft(kpad)) / (n1 n2)
    void* spec = nullptr;   // work spectrum
    void* field = nullptr;  // real field, packed n1 x n2
    SpecConv* sc = nullptr;  // this library's transforms (sides of 2, 3 and 5), else cuFFT
    int nsm = 148;
};

template <typename T> struct FftTypes;
template <> struct FftTypes<float> {
    using C = cufftComplex;
    static constexpr cufftType R2C = CUFFT_R2C, C2R = CUFFT_C2R;
    static cufftResult fwd(cufftHandle h, const float* in, C* out) { return cufftExecR2C(h, (cufftReal*)in, out); }
    static cufftResult inv(cufftHandle h, C* in, float* out) { return cufftExecC2R(h, in, out); }
};
template <> struct FftTypes<double> {
    using C = cufftDoubleComplex;
    static constexpr cufftType R2C = CUFFT_D2Z, C2R = CUFFT_Z2D;
    static cufftResult fwd(cufftHandle h, const double* in, C* out) {
        return cufftExecD2Z(h, (cufftDoubleReal*)in, out);
    }
    static cufftResult inv(cufftHandle h, C* in, double* out) { return cufftExecZ2D(h, in, out); }
};

// The FFTW extension's kernel spectrum (ext/CellularAutomataCoreFFTWExt.jl:17-23): the
// weight of offset o added at mod1(o + 1, dims) — 0-based (o mod n) — transformed once,
// conjugated, with cuFFT's missing 1/(n1 n2) of the inverse folded in.
template <typename T>
int fft_setup(LeniaPlan* P, cudaStream_t st, std::string& err) {
    using F = FftTypes<T>;
    using C = typename F::C;
    const int64_t n1 = P->n1, n2 = P->n2, nc = n1 / 2 + 1;
    const int ntaps = (int)P->w.size();
    std::vector<T> kpad((size_t)(n1 * n2), T(0));
    for (int k = 0; k < ntaps; ++k) {
        const int64_t a = map_axis(GBCA_PERIODIC, P->off[2 * k], n1), b = map_axis(GBCA_PERIODIC, P->off[2 * k + 1], n2);
        kpad[(size_t)(a + b * n1)] += (T)P->w[k];
    }
    int dims[2] = {(int)n2, (int)n1};
    int inembed[2] = {(int)n2, (int)P->pe};
    int fembed[2] = {(int)n2, (int)n1};
    int cembed[2] = {(int)n2, (int)nc};
    cufftResult r = cufftPlanMany(&P->fwd, 2, dims, inembed, 1, (int)(P->pe * n2), cembed, 1, (int)(nc * n2), F::R2C, 1);
    if (r == CUFFT_SUCCESS)
        r = cufftPlanMany(&P->inv, 2, dims, cembed, 1, (int)(nc * n2), fembed, 1, (int)(n1 * n2), F::C2R, 1);
    if (r != CUFFT_SUCCESS) return fail_to(err, GBCA_ERR_CUDA, "cuFFT plan creation failed");
    cudaError_t e = cudaMalloc(&P->kspec, sizeof(C) * nc * n2);
    if (e == cudaSuccess) e = cudaMalloc(&P->spec, sizeof(C) * nc * n2);
    if (e == cudaSuccess) e = cudaMalloc(&P->field, sizeof(T) * n1 * n2);
    if (e != cudaSuccess) return fail_to(err, GBCA_ERR_OUT_OF_MEMORY, cudaGetErrorString(e));
    // transform kpad with the inverse plan's layout (packed input)
    cufftHandle kplan = 0;
    T* d_kpad = nullptr;
    e = cudaMalloc(&d_kpad, sizeof(T) * n1 * n2);
    if (e == cudaSuccess) e = cudaMemcpyAsync(d_kpad, kpad.data(), sizeof(T) * n1 * n2, cudaMemcpyHostToDevice, st);
    if (e == cudaSuccess) r = cufftPlanMany(&kplan, 2, dims, fembed, 1, (int)(n1 * n2), cembed, 1, (int)(nc * n2), F::R2C, 1);
    if (e == cudaSuccess && r == CUFFT_SUCCESS) r = cufftSetStream(kplan, st);
    if (e == cudaSuccess && r == CUFFT_SUCCESS) r = F::fwd(kplan, d_kpad, (C*)P->kspec);
    std::vector<C> ks;
    if (e == cudaSuccess && r == CUFFT_SUCCESS) {
        ks.resize((size_t)(nc * n2));
        e = cudaMemcpyAsync(ks.data(), P->kspec, sizeof(C) * nc * n2, cudaMemcpyDeviceToHost, st);
        if (e == cudaSuccess) e = cudaStreamSynchronize(st);
    }
    if (kplan) cufftDestroy(kplan);
    cudaFree(d_kpad);
    if (r != CUFFT_SUCCESS) return fail_to(err, GBCA_ERR_CUDA, "cuFFT transform of the kernel failed");
    if (e != cudaSuccess) return fail_to(err, GBCA_ERR_CUDA, cudaGetErrorString(e));
    const T scale = T(1) / (T)(n1 * n2);
    for (auto& c : ks) {
        c.x *= scale;
        c.y = -c.y * scale;
    }
    e = cudaMemcpyAsync(P->kspec, ks.data(), sizeof(C) * nc * n2, cudaMemcpyHostToDevice, st);
    if (e == cudaSuccess) e = cudaStreamSynchronize(st);
    if (e != cudaSuccess) return fail_to(err, GBCA_ERR_CUDA, cudaGetErrorString(e));
    return GBCA_OK;
}

int lenia_create(const gbca_desc& d, int64_t pitch_bytes, cudaStream_t st, LeniaPlan** out, std::string& err) {
    *out = nullptr;
    LeniaPlan* P = new LeniaPlan();
    P->d = d;
    P->n1 = d.n1;
    P->n2 = d.n2;
    P->f64 = d.lenia_f64 != 0;
    const int64_t es = P->f64 ? 8 : 4;
    P->pe = pitch_bytes / es;
    P->fft = d.lenia_method == GBCA_FFT;
    int dev = 0;
    cudaGetDevice(&dev);
    cudaDeviceGetAttribute(&P->nsm, cudaDevAttrMultiProcessorCount, dev);
    // kernel_weights (kernels.jl:174-189): column-major offsets, d <= R + 1e-9, w > 0,
    // normalised in FP64; environment.jl:62 negates the offsets.
    const int R = d.lenia_R;
    for (int dj = -R; dj <= R; ++dj)
        for (int di = -R; di <= R; ++di) {
            const double dist = std::sqrt((double)(di * di + dj * dj));
            if (!(dist <= (double)R + 1e-9)) continue;
            const double v = lenia_value(dist, R, d.lenia_peaks, d.lenia_npeaks);
            if (v > 0.0) {
                P->off.push_back(-di);
                P->off.push_back(-dj);
                P->w.push_back(v);
            }
        }
    if (P->w.empty()) {
        delete P;
        return fail_to(err, GBCA_ERR_ARGUMENT, "the Lenia kernel has no positive weight on this lattice");
    }
    double sum = 0.0;
    for (double v : P->w) sum += v;
    for (double& v : P->w) v /= sum;
    const int ntaps = (int)P->w.size();

    // the specialised R = 13 kernel needs exactly the open disk as its tap set
    P->box13 = R == kR13;
    std::memset(&P->b32, 0, sizeof P->b32);
    std::memset(&P->b64, 0, sizeof P->b64);
    if (P->box13) {
        int disk = 0;
        for (int dj = -kR13; dj <= kR13; ++dj)
            for (int di = -kR13; di <= kR13; ++di) disk += in_disk13(di, dj);
        if (disk != ntaps) P->box13 = false;
        for (int k = 0; k < ntaps && P->box13; ++k) {
            const int di = P->off[2 * k], dj = P->off[2 * k + 1];
            if (!in_disk13(di, dj)) P->box13 = false;
            P->b32.w[(dj + kR13) * kBox13 + di + kR13] = (float)P->w[k];
            P->b64.w[(dj + kR13) * kBox13 + di + kR13] = P->w[k];
        }
        // the kernel pairs rows dj and -dj: their weights must be equal (a radial kernel's are)
        for (int dj = 1; dj <= kR13 && P->box13; ++dj)
            for (int di = -kR13; di <= kR13; ++di)
                if (P->b64.w[(dj + kR13) * kBox13 + di + kR13] != P->b64.w[(kR13 - dj) * kBox13 + di + kR13])
                    P->box13 = false;
    }
    cudaError_t e = cudaMalloc(&P->d_off, sizeof(int2) * ntaps);
    if (e == cudaSuccess) e = cudaMalloc(&P->d_w, (size_t)es * ntaps);
    if (e == cudaSuccess) {
        std::vector<float> w32(P->w.begin(), P->w.end());
        e = cudaMemcpyAsync(P->d_off, P->off.data(), sizeof(int2) * ntaps, cudaMemcpyHostToDevice, st);
        if (e == cudaSuccess)
            e = cudaMemcpyAsync(P->d_w, P->f64 ? (const void*)P->w.data() : (const void*)w32.data(), (size_t)es * ntaps,
                                cudaMemcpyHostToDevice, st);
        if (e == cudaSuccess) e = cudaStreamSynchronize(st);
    }
    if (e != cudaSuccess) {
        lenia_destroy(P);
        return fail_to(err, GBCA_ERR_CUDA, cudaGetErrorString(e));
    }

    if (P->fft && specconv_supported(P->n1, P->n2, P->f64)) {
        // kpad at 0-based (o mod n) per axis, each weight in the state's precision (environment.jl:63)
        std::vector<double> kpad((size_t)(P->n1 * P->n2), 0.0);
        for (int k = 0; k < ntaps; ++k) {
            const int64_t a = map_axis(GBCA_PERIODIC, P->off[2 * k], P->n1);
            const int64_t b = map_axis(GBCA_PERIODIC, P->off[2 * k + 1], P->n2);
            kpad[(size_t)(a + b * P->n1)] += P->f64 ? P->w[k] : (double)(float)P->w[k];
        }
        const int rc = specconv_create(P->n1, P->n2, P->f64, kpad.data(), st, &P->sc, err);
        if (rc != GBCA_OK) {
            lenia_destroy(P);
            return rc;
        }
    } else if (P->fft) {
        const int rc = P->f64 ? fft_setup<double>(P, st, err) : fft_setup<float>(P, st, err);
        if (rc != GBCA_OK) {
            lenia_destroy(P);
            return rc;
        }
    }
    *out = P;
    return GBCA_OK;
}

void lenia_destroy(LeniaPlan* P) {
    if (!P) return;
    if (P->fwd) cufftDestroy(P->fwd);
    if (P->inv) cufftDestroy(P->inv);
    specconv_destroy(P->sc);
    cudaFree(P->d_off);
    cudaFree(P->d_w);
    cudaFree(P->kspec);
    cudaFree(P->spec);
    cudaFree(P->field);
    delete P;
}

template <typename T>
int advance_t(LeniaPlan* P, int64_t nsteps, cudaStream_t st, int* cur, void* const bufs[2], std::string& err) {
    using F = FftTypes<T>;
    using C = typename F::C;
    const T mu = (T)P->d.lenia_mu, sigma = (T)P->d.lenia_sigma, dt = (T)P->d.lenia_dt;
    const int b1 = P->d.boundary[0], b2 = P->d.boundary[1];
    if (P->sc) {  // this library's transforms: the whole run, steps chained
        const cudaError_t e = specconv_lenia_run(P->sc, bufs, cur, nsteps, P->pe, P->d.lenia_mu, P->d.lenia_sigma,
                                                 P->d.lenia_dt, st);
        return e == cudaSuccess ? GBCA_OK : fail_to(err, GBCA_ERR_CUDA, cudaGetErrorString(e));
    }
    for (int64_t s = 0; s < nsteps; ++s) {
        const T* u = (const T*)bufs[*cur];
        T* out = (T*)bufs[*cur ^ 1];
        cudaError_t e = cudaSuccess;
        if (P->fft) {
            const int64_t nc = P->n1 / 2 + 1;
            if (cufftSetStream(P->fwd, st) != CUFFT_SUCCESS || cufftSetStream(P->inv, st) != CUFFT_SUCCESS ||
                F::fwd(P->fwd, u, (C*)P->spec) != CUFFT_SUCCESS)
                return fail_to(err, GBCA_ERR_CUDA, "cuFFT forward transform failed");
            k_spectral_mul<C><<<P->nsm * 8, 256, 0, st>>>((C*)P->spec, (const C*)P->kspec, nc * P->n2);
            if (F::inv(P->inv, (C*)P->spec, (T*)P->field) != CUFFT_SUCCESS)
                return fail_to(err, GBCA_ERR_CUDA, "cuFFT inverse transform failed");
            k_growth<T><<<P->nsm * 8, 256, 0, st>>>(u, (const T*)P->field, out, P->n1, P->n2, P->pe, P->n1, mu, sigma,
                                                    dt);
            count_launch(2);
        } else if (P->box13) {
            constexpr int sy = kDirTY + 2 * kR13, sp = lenia13_pitch<T>();
            const Box13<T>* wb;
            if constexpr (sizeof(T) == 4) wb = &P->b32;
            else wb = &P->b64;
            const int tiles_x = (int)((P->n1 + kDirTX - 1) / kDirTX), tiles_y = (int)((P->n2 + kDirTY - 1) / kDirTY);
            const size_t smem = 2 * sizeof(T) * sp * sy;
            e = ensure_dynamic_smem((const void*)k_lenia13p<T>, smem);
            if (e != cudaSuccess) return fail_to(err, GBCA_ERR_CUDA, cudaGetErrorString(e));
            int per_sm = 0;
            e = cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, k_lenia13p<T>, (kDirTX / kDirCells) * kDirTY,
                                                              smem);
            if (e != cudaSuccess) return fail_to(err, GBCA_ERR_CUDA, cudaGetErrorString(e));
            const int ntiles = tiles_x * tiles_y;
            int blocks = P->nsm * (per_sm > 0 ? per_sm : 1);
            if (blocks > ntiles) blocks = ntiles;
            k_lenia13p<T><<<blocks, (kDirTX / kDirCells) * kDirTY, smem, st>>>(u, out, P->n1, P->n2, P->pe, b1, b2,
                                                                               *wb, mu, sigma, dt, tiles_x, ntiles);
            count_launch();
        } else {
            const int R = P->d.lenia_R, tile = 32;
            const size_t smem = sizeof(T) * (tile + 2 * R) * (tile + 2 * R);
            e = ensure_dynamic_smem((const void*)k_lenia_taps<T>, smem);
            if (e != cudaSuccess) return fail_to(err, GBCA_ERR_CUDA, cudaGetErrorString(e));
            dim3 grid((unsigned)((P->n1 + tile - 1) / tile), (unsigned)((P->n2 + tile - 1) / tile));
            k_lenia_taps<T><<<grid, 256, smem, st>>>(u, out, P->n1, P->n2, P->pe, b1, b2, P->d_off, (const T*)P->d_w,
                                                     (int)P->w.size(), R, mu, sigma, dt);
            count_launch();
        }
        e = cudaGetLastError();
        if (e != cudaSuccess) return fail_to(err, GBCA_ERR_CUDA, cudaGetErrorString(e));
        *cur ^= 1;
    }
    return GBCA_OK;
}

int lenia_advance(LeniaPlan* P, int64_t nsteps, cudaStream_t st, int* cur, void* const bufs[2], std::string& err) {
    if (!P) return fail_to(err, GBCA_ERR_ARGUMENT, "no Lenia plan");
    return P->f64 ? advance_t<double>(P, nsteps, st, cur, bufs, err) : advance_t<float>(P, nsteps, st, cur, bufs, err);
}

}  // namespace gbca
