// measures.cu — state_counts (src/measures.jl:14-20) and Moran's I with VonNeumann(1)
// (src/measures.jl:91-107) on an Int8 state in HBM, as exact integer sums.
//
// Moran's I is  n/W * sum_i sum_{j in N(i)} (x_i - m)(x_j - m) / sum_i (x_i - m)^2  with
// m = S/n. Expanding the products, it is a ratio of integers,
//   (n^2 P - n S Q + W S^2) / (W (n S2 - S^2)),
// where S = sum x, S2 = sum x^2, P = sum over neighbour pairs of x_i x_j, Q = sum over
// pairs of (x_i + x_j) and W the number of pairs. The kernel accumulates those integers
// (order-independent, so every launch shape gives the same bits); the host finishes the
// ratio in 128-bit integers and divides once.
#include <atomic>

#include "gbca_internal.cuh"
#include "measures.cuh"

namespace gbca {

namespace {

__global__ void __launch_bounds__(256) k_measures(const int8_t* __restrict__ u, int64_t n1, int64_t n2,
                                                  int64_t pitch, int32_t b1, int32_t b2, int64_t j_lo, int64_t j_hi,
                                                  unsigned long long* __restrict__ acc) {
    __shared__ unsigned int hist[256];
    __shared__ long long sums[5];
    for (int k = threadIdx.x; k < 256; k += blockDim.x) hist[k] = 0;
    if (threadIdx.x < 5) sums[threadIdx.x] = 0;
    __syncthreads();
    long long S = 0, S2 = 0, P = 0, Q = 0, W = 0;
    const int64_t n = n1 * (j_hi - j_lo);  // the cells of columns j_lo .. j_hi - 1
    for (int64_t k = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; k < n; k += (int64_t)gridDim.x * blockDim.x) {
        const int64_t i = k % n1, j = j_lo + k / n1;
        const int x = u[i + j * pitch];
        atomicAdd(&hist[x + 128], 1u);
        S += x;
        S2 += x * x;
        // VonNeumann(1) offsets in the reference's order: (0,-1), (-1,0), (1,0), (0,1)
        const int di[4] = {0, -1, 1, 0}, dj[4] = {-1, 0, 0, 1};
#pragma unroll
        for (int q = 0; q < 4; ++q) {
            const int64_t a = map_axis(b1, i + di[q], n1), b = map_axis(b2, j + dj[q], n2);
            if (a < 0 || b < 0) continue;  // beyond a Constant edge: not a neighbour
            const int y = u[a + b * pitch];
            P += x * y;
            Q += x + y;
            W += 1;
        }
    }
    // warp reduction, then one atomic per warp into shared, one per block into global
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) {
        S += __shfl_down_sync(0xffffffffu, S, o);
        S2 += __shfl_down_sync(0xffffffffu, S2, o);
        P += __shfl_down_sync(0xffffffffu, P, o);
        Q += __shfl_down_sync(0xffffffffu, Q, o);
        W += __shfl_down_sync(0xffffffffu, W, o);
    }
    if ((threadIdx.x & 31) == 0) {
        atomicAdd((unsigned long long*)&sums[0], (unsigned long long)S);
        atomicAdd((unsigned long long*)&sums[1], (unsigned long long)S2);
        atomicAdd((unsigned long long*)&sums[2], (unsigned long long)P);
        atomicAdd((unsigned long long*)&sums[3], (unsigned long long)Q);
        atomicAdd((unsigned long long*)&sums[4], (unsigned long long)W);
    }
    __syncthreads();
    for (int k = threadIdx.x; k < 256; k += blockDim.x)
        if (hist[k]) atomicAdd(&acc[k], (unsigned long long)hist[k]);
    if (threadIdx.x < 5) atomicAdd(&acc[256 + threadIdx.x], (unsigned long long)sums[threadIdx.x]);
}

}  // namespace

namespace {

__global__ void k_soup(int8_t* __restrict__ buf, int64_t n1, int64_t n2, int64_t pitch, uint64_t seed, uint32_t thr24) {
    const int64_t n = n1 * n2;
    for (int64_t q = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; q < n; q += (int64_t)gridDim.x * blockDim.x) {
        const uint2 w = cell_draw(seed, (uint64_t)q + 1u, (int64_t)0xFFFFFFFFu, 0xFFFFFFFEu);
        buf[(q % n1) + (q / n1) * pitch] = (int8_t)((w.x >> 8) < thr24 ? 1 : 0);
    }
}

}  // namespace

cudaError_t launch_soup(int8_t* buf, int64_t n1, int64_t n2, int64_t pitch, double density, uint64_t seed, int grid,
                        cudaStream_t st) {
    const uint32_t thr = (uint32_t)gbca_threshold(density, 1);
    k_soup<<<grid, 256, 0, st>>>(buf, n1, n2, pitch, seed, thr);
    count_launch();
    return cudaGetLastError();
}

cudaError_t launch_measures(const int8_t* u, int64_t n1, int64_t n2, int64_t pitch, int32_t b1, int32_t b2,
                            unsigned long long* acc, int nsm, cudaStream_t st, int64_t j_lo, int64_t j_hi) {
    cudaError_t e = cudaMemsetAsync(acc, 0, kMeasureWords * sizeof(unsigned long long), st);
    if (e != cudaSuccess) return e;
    if (j_hi < 0) j_hi = n2;
    const int64_t n = n1 * (j_hi - j_lo);
    int64_t blocks = (n + 255) / 256;
    const int64_t cap = (int64_t)nsm * 8;
    if (blocks > cap) blocks = cap;
    if (blocks < 1) blocks = 1;
    k_measures<<<(unsigned)blocks, 256, 0, st>>>(u, n1, n2, pitch, b1, b2, j_lo, j_hi, acc);
    count_launch();
    return cudaGetLastError();
}

namespace {

// Whether every cell of an Int8 state lies in 0 .. nv - 1: 16-byte chunks of each column,
// compared byte by byte as unsigned (a negative value is >= 128), the bytes past n1 ignored.
// Any thread that finds a value outside sets *bad; a warp votes first, so one atomic per warp.
__global__ void __launch_bounds__(256) k_states_in_range(const int8_t* __restrict__ u, int64_t n1, int64_t n2,
                                                         int64_t pitch, uint32_t nv, unsigned int* __restrict__ bad) {
    const int64_t chunks = (n1 + 15) / 16, total = chunks * n2;
    const uint32_t lim = nv * 0x01010101u;
    bool found = false;
    for (int64_t q = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; q < total; q += (int64_t)gridDim.x * blockDim.x) {
        const int64_t c = q % chunks, j = q / chunks;
        const int4 v = *(const int4*)(u + j * pitch + 16 * c);
        const uint32_t w[4] = {(uint32_t)v.x, (uint32_t)v.y, (uint32_t)v.z, (uint32_t)v.w};
        const int64_t inside = n1 - 16 * c;  // bytes of this chunk inside the lattice (>= 1)
#pragma unroll
        for (int k = 0; k < 4; ++k) {
            uint32_t ok = __vcmpltu4(w[k], lim);  // 0xFF in each byte below nv
            const int64_t nb = inside - 4 * k;    // bytes of this word inside the lattice
            if (nb < 4) ok |= nb <= 0 ? 0xFFFFFFFFu : (0xFFFFFFFFu << (8 * nb));
            found = found || ok != 0xFFFFFFFFu;
        }
    }
    if (__any_sync(0xFFFFFFFFu, found) && (threadIdx.x & 31) == 0) atomicOr(bad, 1u);
}

std::atomic<int64_t> g_launches{0};

}  // namespace

cudaError_t launch_states_in_range(const int8_t* u, int64_t n1, int64_t n2, int64_t pitch, int32_t nv,
                                   unsigned int* bad, int nsm, cudaStream_t st) {
    if (pitch % 16 != 0 || ((uintptr_t)u & 15u) != 0 || nv < 1 || nv > 255) return cudaErrorInvalidValue;
    cudaError_t e = cudaMemsetAsync(bad, 0, sizeof(unsigned int), st);
    if (e != cudaSuccess) return e;
    const int64_t total = (n1 + 15) / 16 * n2;
    int64_t blocks = (total + 255) / 256;
    const int64_t cap = (int64_t)nsm * 8;
    if (blocks > cap) blocks = cap;
    if (blocks < 1) blocks = 1;
    k_states_in_range<<<(unsigned)blocks, 256, 0, st>>>(u, n1, n2, pitch, (uint32_t)nv, bad);
    count_launch();
    return cudaGetLastError();
}

void count_launch(int64_t n) { g_launches.fetch_add(n, std::memory_order_relaxed); }
int64_t launches_so_far() { return g_launches.load(std::memory_order_relaxed); }

void finish_measures(const unsigned long long* acc, int64_t n, int64_t* counts, int32_t nvals, int64_t* other,
                     double* morans) {
    int64_t inrange = 0;
    for (int v = 0; v < nvals; ++v) {
        const int64_t c = (v >= 0 && v < 128) ? (int64_t)acc[v + 128] : 0;
        if (counts) counts[v] = c;
        inrange += c;
    }
    if (other) *other = n - inrange;
    if (!morans) return;
    *morans = morans_from_sums((long long)acc[256], (long long)acc[257], (long long)acc[258], (long long)acc[259],
                               (long long)acc[260], n);
}

double morans_from_sums(long long s, long long s2, long long p, long long q, long long w, int64_t n) {
    const __int128 S = s, S2 = s2, P = p, Q = q, W = w, N = n;
    const __int128 num = N * N * P - N * S * Q + W * S * S;
    const __int128 den = W * (N * S2 - S * S);
    if (den == 0 || W == 0) return __builtin_nan("");
    return (double)((long double)num / (long double)den);
}

}  // namespace gbca
