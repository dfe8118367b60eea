// lenia.cuh — Lenia (src/lenia.jl) on the device in Float32 or Float64: direct and FFT kernel fields.
#pragma once
#include <cstdint>
#include <string>
#include <cuda_runtime.h>

#include "gbca.h"

namespace gbca {

struct LeniaPlan;

int lenia_create(const gbca_desc& d, int64_t pitch_bytes, cudaStream_t st, LeniaPlan** out, std::string& err);
void lenia_destroy(LeniaPlan* plan);
// nsteps Lenia steps, ping-ponging between bufs[*cur] and bufs[*cur ^ 1]; updates *cur.
int lenia_advance(LeniaPlan* plan, int64_t nsteps, cudaStream_t st, int* cur, void* const bufs[2], std::string& err);

}  // namespace gbca
