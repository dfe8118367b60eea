// measures.cuh — device summaries of an Int8 state (counts per value, Moran's I sums).
#pragma once
#include <cstdint>
#include <cuda_runtime.h>

namespace gbca {

// Accumulator layout: [0, 256) histogram of value + 128; then S, S2, P, Q, W.
constexpr int kMeasureWords = 261;

// A Bernoulli(density) soup of 0/1 from a seed, on the device: cell id's draw is
// (seed; id, 0, 0xFFFFFFFF, 0xFFFFFFFE), a counter the rules never use, compared as a Float32
// uniform. The synthetic initial state of requests and handles that are given none.
cudaError_t launch_soup(int8_t* buf, int64_t n1, int64_t n2, int64_t pitch, double density, uint64_t seed, int grid,
                        cudaStream_t st);

// The sums over the cells of columns j_lo .. j_hi - 1 (j_hi < 0: through column n2 - 1), their
// neighbours read through the lattice's boundaries: a slab's share of a larger lattice's sums.
cudaError_t launch_measures(const int8_t* u, int64_t n1, int64_t n2, int64_t pitch, int32_t b1, int32_t b2,
                            unsigned long long* acc, int nsm, cudaStream_t st, int64_t j_lo = 0, int64_t j_hi = -1);

// *bad = 0 when every cell of the state lies in 0 .. nv - 1 (nv in 1..255), else nonzero.
// Needs a 16-byte-aligned buffer and pitch; the bytes between n1 and the pitch are not read
// as cells.
cudaError_t launch_states_in_range(const int8_t* u, int64_t n1, int64_t n2, int64_t pitch, int32_t nv,
                                   unsigned int* bad, int nsm, cudaStream_t st);

// counts[v] for v < nvals, *other = cells outside, *morans from the integer sums
// (NaN for a constant field). Any output pointer may be null.
void finish_measures(const unsigned long long* acc, int64_t n, int64_t* counts, int32_t nvals, int64_t* other,
                     double* morans);

// Moran's I from its integer sums (S, S2, P, Q, W) over n cells; NaN for a constant field.
double morans_from_sums(long long S, long long S2, long long P, long long Q, long long W, int64_t n);

}  // namespace gbca
