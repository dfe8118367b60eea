// sweep_field.cu — the kernel-field SI rule: a sweep whose rule reads a dispersal-kernel field
// (src/environment.jl:1-69,151-169) and a covariate (environment.jl:71-113), under a mask
// (environment.jl:123-130, backends.jl:448-450).
//
// The rule is the conformance battery's kernel-field epidemic as a typed rule
// (test/backend_conformance.jl:52-57 with a covariate, :72-75 in Float32): a cell in state 1
// stays 1; any other cell becomes 1 when bernoulli(ctx, 1 - exp(-beta * cov * field)) with
// draw k = 1 (random.jl:129-130), else keeps its state. The field is
// sum_k w_k * source(u[I + o_k]) in tap order (source: u == 1, or u itself), computed from the
// state at the start of the step (backends.jl:481-506), in Float32 or Float64.
//
// One launch per step. A CTA stages its 64 x 32 output tile plus a halo of the kernel's radius
// in shared memory through the boundary mapping, then each thread evaluates its cells. A
// source of 0 adds +0.0, which leaves the running sum unchanged, so only taps that read a
// nonzero source are added (the sum is bit-identical to the full one); a tile whose staged
// region holds no nonzero source has every field exactly 0, hence no infection, and skips
// the tap loop. The rule never reads its neighbours directly and the field is fixed for the
// whole step, so Checkerboard's two half-sweeps update every cell once from the start-of-step
// values: one pass covers both. With method = :fft the field comes from a spectral product
// instead (ext/CellularAutomataCoreFFTWExt.jl:17-30) and the tile needs no halo: this
// library's transforms (spectral.cu) where both sides are products of 2, 3 and 5, cuFFT else.
#include <cmath>
#include <vector>

#include <cufft.h>

#include "field.cuh"
#include "spectral.cuh"
#include "gbca_internal.cuh"

namespace gbca {

namespace {

constexpr int kSiTX = 64, kSiTY = 32, kSiThreads = 256;

// Julia's promotion for a product: Float32 * Float32 stays Float32, anything else is Float64.
struct Num {
    bool f32;
    float f;
    double d;
};
__device__ __forceinline__ Num num32(float f) { return Num{true, f, (double)f}; }
__device__ __forceinline__ Num num64(double d) { return Num{false, (float)d, d}; }
__device__ __forceinline__ Num num_mul(Num a, Num b) {
    if (a.f32 && b.f32) return num32(__fmul_rn(a.f, b.f));
    return num64(__dmul_rn(a.d, b.d));
}

__device__ __forceinline__ bool source_nonzero(int8_t v, int source) {
    return source == kSourceIdentity ? v != 0 : v == 1;
}

template <bool F32>
__device__ __forceinline__ Num direct_field(const FieldSweep& p, const int8_t* S, int sx, int lx, int ly) {
    // lx, ly: the cell's position in the staged region (halo included)
    if (F32) {
        float s = 0.0f;
        for (int k = 0; k < p.ntaps; ++k) {
            const int2 o = __ldg(&p.taps[k]);
            const int8_t v = S[(ly + o.y) * sx + lx + o.x];
            if (source_nonzero(v, p.source)) {
                const float w = __ldg(&p.w32[k]);
                s = __fadd_rn(s, p.source == kSourceIdentity ? __fmul_rn(w, (float)v) : w);
            }
        }
        return num32(s);
    }
    double s = 0.0;
    for (int k = 0; k < p.ntaps; ++k) {
        const int2 o = __ldg(&p.taps[k]);
        const int8_t v = S[(ly + o.y) * sx + lx + o.x];
        if (source_nonzero(v, p.source)) {
            const double w = __ldg(&p.w64[k]);
            s = __dadd_rn(s, p.source == kSourceIdentity ? __dmul_rn(w, (double)v) : w);
        }
    }
    return num64(s);
}

// bernoulli(ctx, q, 1) in the precision of q, from its exact integer threshold.
__device__ __forceinline__ bool bernoulli_q(const FieldSweep& p, uint64_t id, Num q) {
    uint64_t thr;
    if (q.f32) {
        if (!(q.f > 0.0f)) return false;
        if (q.f >= 1.0f) return true;
        thr = (uint64_t)ceil((double)q.f * 16777216.0);
    } else {
        if (!(q.d > 0.0)) return false;
        if (q.d >= 1.0) return true;
        thr = (uint64_t)ceil(q.d * 9007199254740992.0);
    }
    return draw_below(cell_draw(p.seed, id, p.t, 1), thr, q.f32);
}

template <bool F32>
__global__ void __launch_bounds__(kSiThreads) k_si(FieldSweep p, const int8_t* __restrict__ src,
                                                   int8_t* __restrict__ dst) {
    extern __shared__ int8_t S[];
    const int R = p.field ? 0 : p.R;
    const int sx = kSiTX + 2 * R, sy = kSiTY + 2 * R;
    const int64_t X0 = (int64_t)blockIdx.x * kSiTX, Y0 = (int64_t)blockIdx.y * kSiTY;
    int any = 0;
    for (int q = threadIdx.x; q < sx * sy; q += blockDim.x) {
        const int lx = q % sx, ly = q / sx;
        const int64_t mx = map_axis(p.bnd[0], X0 - R + lx, p.n1), my = map_axis(p.bnd[1], Y0 - R + ly, p.n2);
        int8_t v;
        if (my < 0) v = (int8_t)p.cval[1];
        else if (mx < 0) v = (int8_t)p.cval[0];
        else v = src[mx + my * p.pitch];
        S[q] = v;
        any |= source_nonzero(v, p.source);
    }
    any = __syncthreads_or(any);
    for (int q = threadIdx.x; q < kSiTX * kSiTY; q += blockDim.x) {
        const int lx = q % kSiTX, ly = q / kSiTX;
        const int64_t gx = X0 + lx, gy = Y0 + ly;
        if (gx >= p.n1 || gy >= p.n2) continue;
        const int8_t c = S[(ly + R) * sx + lx + R];
        int8_t out = c;
        const bool frozen = p.mask && !p.mask[gx + gy * p.pitch];
        if (!frozen && c != 1 && (any || p.field)) {
            Num f;
            if (p.field) f = F32 ? num32(((const float*)p.field)[gx + gy * p.n1])
                                 : num64(((const double*)p.field)[gx + gy * p.n1]);
            else f = direct_field<F32>(p, S, sx, lx + R, ly + R);
            if (f.d != 0.0) {  // a zero field never infects (q = 0, or NaN)
                Num lam = p.beta_f32 ? num32((float)p.beta) : num64(p.beta);
                if (p.cov) {
                    const int64_t at = gx + gy * p.n1 + p.cov_slice * p.n1 * p.n2;
                    lam = num_mul(lam, p.cov_f32 ? num32(((const float*)p.cov)[at]) : num64(((const double*)p.cov)[at]));
                }
                lam = num_mul(lam, f);
                Num qv;
                if (lam.f32) qv = num32(__fsub_rn(1.0f, (float)exp(-(double)lam.f)));
                else qv = num64(__dsub_rn(1.0, exp(-lam.d)));
                const uint64_t id = (uint64_t)gx + (uint64_t)gy * (uint64_t)p.n1 + 1u;
                if (bernoulli_q(p, id, qv)) {
                    bool open = true;  // src/schemes.jl:84-89 (Checkerboard: every cell once)
                    if (p.scheme == GBCA_STOCHASTIC)
                        open = draw_below(cell_draw(p.seed, id, p.t, 0), p.gate_thr, p.gate_f32);
                    if (open) out = 1;
                }
            }
        }
        dst[gx + gy * p.pitch] = out;
    }
}

// ---------------------------------------------------------------- FFT fields

__global__ void k_source(const int8_t* __restrict__ u, int64_t n1, int64_t n2, int64_t pitch, int source,
                         bool f32, void* __restrict__ out) {
    const int64_t n = n1 * n2;
    for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x) {
        const int8_t v = u[(i % n1) + (i / n1) * pitch];
        const double x = source == kSourceIdentity ? (double)v : (v == 1 ? 1.0 : 0.0);
        if (f32) ((float*)out)[i] = (float)x;
        else ((double*)out)[i] = x;
    }
}

template <typename C>
__global__ void k_cmul(C* __restrict__ a, const C* __restrict__ k, int64_t n) {
    for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x) {
        const C x = a[i], y = k[i];
        a[i] = C{x.x * y.x - x.y * y.y, x.x * y.y + x.y * y.x};
    }
}

}  // namespace

struct FieldFFT {
    bool f32 = false;
    int64_t n1 = 0, n2 = 0;
    cufftHandle fwd = 0, inv = 0;
    void* src = nullptr;    // real source array, packed n1 x n2
    void* spec = nullptr;   // its spectrum
    void* kspec = nullptr;  // conj(rfft(kpad)) / (n1 n2)
    void* field = nullptr;  // the real field, packed n1 x n2
    SpecConv* sc = nullptr;  // this library's transforms (sides of 2, 3 and 5); else the cuFFT plans
};

void field_fft_destroy(FieldFFT* F) {
    if (!F) return;
    if (F->fwd) cufftDestroy(F->fwd);
    if (F->inv) cufftDestroy(F->inv);
    specconv_destroy(F->sc);
    cudaFree(F->src);
    cudaFree(F->spec);
    cudaFree(F->kspec);
    cudaFree(F->field);
    delete F;
}

// The FFTW extension's product (ext/CellularAutomataCoreFFTWExt.jl:17-30): the weight of
// offset o added to kpad at 0-based (o mod n) on each axis, transformed once, conjugated,
// with the inverse's 1/(n1 n2) folded in; by spectral.cu where the sides allow, else by cuFFT.
int field_fft_create(int64_t n1, int64_t n2, const std::vector<int>& taps, const std::vector<double>& w, bool f32,
                     cudaStream_t st, FieldFFT** out, std::string& err) {
    *out = nullptr;
    FieldFFT* F = new FieldFFT();
    F->f32 = f32;
    F->n1 = n1;
    F->n2 = n2;
    const int64_t nc = n1 / 2 + 1, n = n1 * n2;
    const size_t es = f32 ? sizeof(float) : sizeof(double), cs = 2 * es;
    if (specconv_supported(n1, n2, !f32)) {  // kpad in FP64, each weight in the field's precision
        std::vector<double> kpad((size_t)n, 0.0);
        for (size_t k = 0; k < w.size(); ++k) {
            const int64_t a = map_axis(GBCA_PERIODIC, taps[2 * k], n1), b = map_axis(GBCA_PERIODIC, taps[2 * k + 1], n2);
            kpad[(size_t)(a + b * n1)] += f32 ? (double)(float)w[k] : w[k];
        }
        int rc = specconv_create(n1, n2, !f32, kpad.data(), st, &F->sc, err);
        if (rc == GBCA_OK && cudaMalloc(&F->field, es * n) != cudaSuccess) {
            err = "out of device memory for the field";
            rc = GBCA_ERR_OUT_OF_MEMORY;
        }
        if (rc != GBCA_OK) {
            field_fft_destroy(F);
            cudaGetLastError();
            return rc;
        }
        *out = F;
        return GBCA_OK;
    }
    int dims[2] = {(int)n2, (int)n1};
    int rembed[2] = {(int)n2, (int)n1};
    int cembed[2] = {(int)n2, (int)nc};
    const cufftType r2c = f32 ? CUFFT_R2C : CUFFT_D2Z, c2r = f32 ? CUFFT_C2R : CUFFT_Z2D;
    cufftResult r = cufftPlanMany(&F->fwd, 2, dims, rembed, 1, (int)n, cembed, 1, (int)(nc * n2), r2c, 1);
    if (r == CUFFT_SUCCESS) r = cufftPlanMany(&F->inv, 2, dims, cembed, 1, (int)(nc * n2), rembed, 1, (int)n, c2r, 1);
    if (r == CUFFT_SUCCESS) r = cufftSetStream(F->fwd, st);
    if (r == CUFFT_SUCCESS) r = cufftSetStream(F->inv, st);
    if (r != CUFFT_SUCCESS) {
        field_fft_destroy(F);
        err = "cuFFT plan creation failed";
        return GBCA_ERR_CUDA;
    }
    cudaError_t e = cudaMalloc(&F->src, es * n);
    if (e == cudaSuccess) e = cudaMalloc(&F->field, es * n);
    if (e == cudaSuccess) e = cudaMalloc(&F->spec, cs * nc * n2);
    if (e == cudaSuccess) e = cudaMalloc(&F->kspec, cs * nc * n2);
    // kpad in the source buffer, transformed into kspec
    std::vector<double> kpad((size_t)n, 0.0);
    for (size_t k = 0; k < w.size(); ++k) {
        const int64_t a = map_axis(GBCA_PERIODIC, taps[2 * k], n1), b = map_axis(GBCA_PERIODIC, taps[2 * k + 1], n2);
        kpad[(size_t)(a + b * n1)] += f32 ? (double)(float)w[k] : w[k];
    }
    std::vector<float> kpad32;
    if (f32) kpad32.assign(kpad.begin(), kpad.end());
    if (e == cudaSuccess)
        e = cudaMemcpyAsync(F->src, f32 ? (const void*)kpad32.data() : (const void*)kpad.data(), es * n,
                            cudaMemcpyHostToDevice, st);
    if (e == cudaSuccess) {
        r = f32 ? cufftExecR2C(F->fwd, (cufftReal*)F->src, (cufftComplex*)F->kspec)
                : cufftExecD2Z(F->fwd, (cufftDoubleReal*)F->src, (cufftDoubleComplex*)F->kspec);
    }
    std::vector<double> ks;
    std::vector<float> ks32;
    if (e == cudaSuccess && r == CUFFT_SUCCESS) {
        if (f32) ks32.resize((size_t)(2 * nc * n2));
        else ks.resize((size_t)(2 * nc * n2));
        e = cudaMemcpyAsync(f32 ? (void*)ks32.data() : (void*)ks.data(), F->kspec, cs * nc * n2,
                            cudaMemcpyDeviceToHost, st);
        if (e == cudaSuccess) e = cudaStreamSynchronize(st);
    }
    if (e == cudaSuccess && r == CUFFT_SUCCESS) {
        const double scale = 1.0 / (double)n;
        for (int64_t i = 0; i < nc * n2; ++i) {
            if (f32) {
                ks32[2 * i] = (float)(ks32[2 * i] * scale);
                ks32[2 * i + 1] = (float)(-ks32[2 * i + 1] * scale);
            } else {
                ks[2 * i] *= scale;
                ks[2 * i + 1] = -ks[2 * i + 1] * scale;
            }
        }
        e = cudaMemcpyAsync(F->kspec, f32 ? (const void*)ks32.data() : (const void*)ks.data(), cs * nc * n2,
                            cudaMemcpyHostToDevice, st);
        if (e == cudaSuccess) e = cudaStreamSynchronize(st);
    }
    if (r != CUFFT_SUCCESS || e != cudaSuccess) {
        err = r != CUFFT_SUCCESS ? "cuFFT transform of the kernel failed" : cudaGetErrorString(e);
        const bool oom = e == cudaErrorMemoryAllocation;
        field_fft_destroy(F);
        cudaGetLastError();
        return oom ? GBCA_ERR_OUT_OF_MEMORY : GBCA_ERR_CUDA;
    }
    *out = F;
    return GBCA_OK;
}

// The field of the current state into F->field.
static cudaError_t field_fft_run(FieldFFT* F, const int8_t* u, int64_t pitch, int source, int nsm, cudaStream_t st) {
    if (F->sc)
        return specconv_field(F->sc, u, pitch, source == kSourceIdentity ? kSpecValue : kSpecIsOne, F->field, st);
    const int64_t nc = F->n1 / 2 + 1;
    const int grid = nsm * 8;
    // the handle's stream may have changed since the plans were made
    if (cufftSetStream(F->fwd, st) != CUFFT_SUCCESS || cufftSetStream(F->inv, st) != CUFFT_SUCCESS)
        return cudaErrorUnknown;
    k_source<<<grid, 256, 0, st>>>(u, F->n1, F->n2, pitch, source, F->f32, F->src);
    count_launch();
    cufftResult r = F->f32 ? cufftExecR2C(F->fwd, (cufftReal*)F->src, (cufftComplex*)F->spec)
                           : cufftExecD2Z(F->fwd, (cufftDoubleReal*)F->src, (cufftDoubleComplex*)F->spec);
    if (r != CUFFT_SUCCESS) return cudaErrorUnknown;
    if (F->f32) k_cmul<cufftComplex><<<grid, 256, 0, st>>>((cufftComplex*)F->spec, (const cufftComplex*)F->kspec, nc * F->n2);
    else
        k_cmul<cufftDoubleComplex>
            <<<grid, 256, 0, st>>>((cufftDoubleComplex*)F->spec, (const cufftDoubleComplex*)F->kspec, nc * F->n2);
    count_launch();
    r = F->f32 ? cufftExecC2R(F->inv, (cufftComplex*)F->spec, (cufftReal*)F->field)
               : cufftExecZ2D(F->inv, (cufftDoubleComplex*)F->spec, (cufftDoubleReal*)F->field);
    if (r != CUFFT_SUCCESS) return cudaErrorUnknown;
    return cudaGetLastError();
}

size_t si_smem_bytes(int R) { return (size_t)(kSiTX + 2 * R) * (size_t)(kSiTY + 2 * R); }

cudaError_t sweep_si(FieldSweep p, FieldFFT* fft, int8_t* const bufs[2], int* cur, int64_t t, int64_t nsteps,
                     int nsm, cudaStream_t st) {
    const dim3 grid((unsigned)((p.n1 + kSiTX - 1) / kSiTX), (unsigned)((p.n2 + kSiTY - 1) / kSiTY));
    const size_t smem = si_smem_bytes(fft ? 0 : p.R);
    cudaError_t e = cudaSuccess;
    if (smem > 48 * 1024) {
        e = cudaFuncSetAttribute(p.field_f32 ? k_si<true> : k_si<false>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                 (int)smem);
        if (e != cudaSuccess) return e;
    }
    for (int64_t s = 0; s < nsteps; ++s) {
        p.t = t + s;
        const int64_t nt = p.cov_nt > 0 ? p.cov_nt : 1;
        p.cov_slice = ((p.t % nt) + nt) % nt;  // mod1(t + 1, nt) - 1
        const int8_t* src = bufs[*cur];
        if (fft) {
            e = field_fft_run(fft, src, p.pitch, p.source, nsm, st);
            if (e != cudaSuccess) return e;
            p.field = fft->field;
        }
        if (p.field_f32) k_si<true><<<grid, kSiThreads, smem, st>>>(p, src, bufs[*cur ^ 1]);
        else k_si<false><<<grid, kSiThreads, smem, st>>>(p, src, bufs[*cur ^ 1]);
        e = cudaGetLastError();
        if (e != cudaSuccess) return e;
        count_launch();
        *cur ^= 1;
    }
    return cudaSuccess;
}

}  // namespace gbca
