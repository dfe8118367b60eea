// spectral.cuh — periodic 2-D convolution of a real n1 x n2 field with a fixed kernel by this
// library's own FFTs: the FFTW extension's field (ext/CellularAutomataCoreFFTWExt.jl:17-30),
// U = irfft(rfft(src) .* conj(rfft(kpad))), for Lenia and for kernel fields on tori.
#pragma once
#include <cstdint>
#include <string>
#include <cuda_runtime.h>

namespace gbca {

struct SpecConv;

// Source of the transformed field: the state's own values (Lenia), or an Int8 state read as
// (x == 1) or as x (a kernel field's source, src/environment.jl:33-58).
enum SpecSource { kSpecReal = 0, kSpecIsOne = 1, kSpecValue = 2 };

// Whether the plan runs this shape: each side a product of 2, 3 and 5, and two lines of the
// longer side fit in shared memory.
bool specconv_supported(int64_t n1, int64_t n2, bool f64);

// A plan for n1 x n2 lattices in Float32 (f64 false) or Float64: kpad holds the kernel wrapped
// on the lattice (n1 * n2 FP64 values, column-major), transformed once in FP64.
int specconv_create(int64_t n1, int64_t n2, bool f64, const double* kpad, cudaStream_t st, SpecConv** out,
                    std::string& err);
void specconv_destroy(SpecConv* p);

// nsteps Lenia steps between bufs[*cur] and bufs[*cur ^ 1] (pitch pe elements), *cur updated:
// each the field by the plan, then clamp(u + dt (2 exp(-(U - mu)^2 / (2 sigma^2)) - 1), 0, 1)
// (src/lenia.jl:42-47); a step's last launch also transforms the new state for the next.
cudaError_t specconv_lenia_run(SpecConv* p, void* const bufs[2], int* cur, int64_t nsteps, int64_t pe, double mu,
                               double sigma, double dt, cudaStream_t st);

// The field of an Int8 state (pitch bytes between columns) into `field` (n1 x n2 packed, the
// plan's precision).
cudaError_t specconv_field(SpecConv* p, const int8_t* u, int64_t pitch, SpecSource src, void* field,
                           cudaStream_t st);

}  // namespace gbca
