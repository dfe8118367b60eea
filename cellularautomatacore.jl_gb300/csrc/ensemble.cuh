// ensemble.cuh — device descriptors and results of the batched ensemble engine.
#pragma once
#include <cstdint>
#include <cuda_runtime.h>

#include "gbca.h"

namespace gbca {

constexpr int kEnsCounts = 8;                  // values 0..7 are counted per instance
constexpr int kEnsSumWords = kEnsCounts + 6;   // counts, cells outside 0..7, S, S2, P, Q, W

// One instance, as the persistent kernel reads it.
struct EnsInstance {
    int64_t n1, n2, pitch;   // lattice dims, bytes between columns
    int64_t off[2];          // byte offsets of its two buffers in the pool
    int64_t t0, nsteps;      // time of the first step and step count of the next run
    uint64_t birth, survive, seed, thr_p, thr_f;
    int32_t rule, nbhd, radius, states;
    int32_t params_f32, bnd0, bnd1, cval0, cval1;
    int32_t cur;             // buffer holding the current state
    int32_t small;           // fits in shared memory with its halo
    int32_t summarize;       // reduce the final state to its summaries at the end of the run
    int32_t depth;           // steps per temporally blocked pass of the tiled path
    int32_t pad_;
};

struct EnsSummary {
    long long w[kEnsSumWords];
};

// The ensemble kernel runs tiles of 64, 128 or 192 cells a side (a template parameter; its
// shared buffers and the small-lattice threshold follow the tile).
bool ensemble_tile_ok(int tile);
// One persistent launch over n instances (order: the queue order); resets the counter first.
cudaError_t launch_ensemble(const EnsInstance* d_inst, const int* d_order, int n, int* d_counter, int8_t* pool,
                            EnsSummary* d_out, int* d_cur, int grid, cudaStream_t st, int tile = 128);
// Grid size that fills the current device with resident CTAs.
int ensemble_grid(int tile = 128);
// Bytes of each of the two shared buffers a CTA of the ensemble kernel has.
int ensemble_smem_cells(int tile = 128);
// Whether an instance runs with its whole lattice (and halo) in shared memory.
bool ensemble_fits_smem(const gbca_desc& d, int tile = 128);
// Steps per pass of the tiled path for a requested depth (0: the deepest the halo allows).
int ensemble_depth(const gbca_desc& d, int depth);
// Whether an instance's rule has the batched multi-CTA pass (launch_fire_batch); such an
// instance of at least the ensemble's large-cell threshold runs there instead of on one CTA of
// the persistent kernel. Instances below kEnsLargeFloor cells never do.
bool ensemble_large_capable(const gbca_desc& d);
constexpr int64_t kEnsLargeFloor = (int64_t)1 << 14;

}  // namespace gbca
