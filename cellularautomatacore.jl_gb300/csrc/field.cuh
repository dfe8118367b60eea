// field.cuh — the kernel-field SI sweep (sweep_field.cu): parameters and entry points.
#pragma once

#include <cstdint>
#include <string>
#include <vector>

#include <cuda_runtime.h>

#include "gbca.h"

namespace gbca {

constexpr int kSourceIndicator = 0;  // source(x) = x == 1
constexpr int kSourceIdentity = 1;   // source(x) = x

// Everything one SI step needs besides the state buffers. Plain data, passed by value.
struct FieldSweep {
    int64_t n1, n2, pitch;
    int32_t bnd[2], cval[2];
    uint64_t seed;
    int64_t t;
    int32_t scheme, gate_f32;
    uint64_t gate_thr;
    const uint8_t* mask;     // nonzero = the cell updates; pitch bytes between columns; or null
    const int2* taps;        // offsets to read (negated kernel offsets), tap order
    const double* w64;       // normalised weights
    const float* w32;        // the same cast to Float32
    int32_t ntaps, R;        // tap count, largest |offset|
    int32_t field_f32;       // the field (weights and sum) is Float32
    int32_t source;          // kSourceIndicator / kSourceIdentity
    const void* cov;         // covariate, packed n1 x n2 x cov_nt (Float64, or Float32), or null
    int64_t cov_nt, cov_slice;
    int32_t cov_f32;
    int32_t beta_f32;        // beta is Float32
    double beta;
    const void* field;       // a precomputed field (packed n1 x n2), or null: direct sum
};

struct FieldFFT;
int field_fft_create(int64_t n1, int64_t n2, const std::vector<int>& taps, const std::vector<double>& w, bool f32,
                     cudaStream_t st, FieldFFT** out, std::string& err);
void field_fft_destroy(FieldFFT* F);

// Shared memory of one SI tile with a halo of R cells.
size_t si_smem_bytes(int R);

// nsteps SI steps from time t, ping-ponging bufs[*cur] / bufs[*cur ^ 1]; fft (or null) computes
// the field by FFT each step.
cudaError_t sweep_si(FieldSweep p, FieldFFT* fft, int8_t* const bufs[2], int* cur, int64_t t, int64_t nsteps,
                     int nsm, cudaStream_t st);

}  // namespace gbca
