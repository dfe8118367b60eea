// noalloc.cu — gbca_advance_noalloc: the Int8 sweep on a state the caller keeps in device
// memory, without allocating anything.
//
// Why: some callers cannot allocate device memory at the moment they need a sweep — code
// that runs while a memory pool owns the whole device (a Julia CuArray pool, a PyTorch
// caching allocator sized to the card), a real-time loop that must not take the allocator's
// locks or wait on it, or a plug-in whose host forbids allocation after start-up.
// gbca_create allocates two state buffers, an accumulator and a stream; this entry point
// allocates none of them. The caller passes the state (it is advanced in place) and a
// stream. The buffer the sweep alternates with is the file-scope device array below, which
// every GPU that loads the library holds until the process exits; states larger than it are
// refused.
//
// Sharing: every call on a device uses the same array, and the array keeps the last call's
// contents. Each sweep pass writes every lattice cell before anything reads it, so nothing
// has to be cleared between calls; but calls that overlap on the GPU (on different streams
// or from different host threads) race on the array. Serialise them.
//
// Set-up: the first call on each device looks up the array's device address with
// cudaGetSymbolAddress, with that device current, and caches it. That first call should come
// before any stream capture on the device.
#include <cmath>
#include <cstdarg>
#include <cstdio>
#include <cstring>
#include <mutex>

#include "gbca_internal.cuh"

namespace gbca {

namespace {

static __device__ __align__(256) int8_t g_noalloc_scratch[GBCA_NOALLOC_SCRATCH_BYTES];

constexpr int kMaxDevices = 64;
std::mutex g_scratch_mutex;
void* g_scratch_addr[kMaxDevices] = {nullptr};

int nfail(int code, const char* fmt, ...) {
    char msg[512];
    va_list ap;
    va_start(ap, fmt);
    vsnprintf(msg, sizeof msg, fmt, ap);
    va_end(ap);
    set_last_error(msg);
    return code;
}

// The device address of the scratch array on the current device (looked up once per device).
cudaError_t scratch_address(void** out) {
    int dev = 0;
    cudaError_t e = cudaGetDevice(&dev);
    if (e != cudaSuccess) return e;
    if (dev < 0 || dev >= kMaxDevices) return cudaErrorInvalidDevice;
    std::lock_guard<std::mutex> lock(g_scratch_mutex);
    if (!g_scratch_addr[dev]) {
        void* p = nullptr;
        e = cudaGetSymbolAddress(&p, g_noalloc_scratch);
        if (e != cudaSuccess) return e;
        g_scratch_addr[dev] = p;
    }
    *out = g_scratch_addr[dev];
    return cudaSuccess;
}

}  // namespace

}  // namespace gbca

extern "C" int gbca_advance_noalloc(const gbca_desc* desc, void* state, int64_t pitch, int64_t t, int64_t nsteps,
                                    const double* params, int32_t nparams, void* stream) {
    using namespace gbca;
    const int rc = gbca_check(desc);  // sets the message itself
    if (rc != GBCA_OK) return rc;
    if (desc->rule == GBCA_RULE_LENIA)
        return nfail(GBCA_ERR_UNSUPPORTED, "gbca_advance_noalloc runs the Int8 rules; Lenia's FFT plans allocate");
    if (desc->rule == GBCA_RULE_SI_FIELD)
        return nfail(GBCA_ERR_UNSUPPORTED, "gbca_advance_noalloc runs no kernel-field rule (its field is set on a handle)");
    if (!state) return nfail(GBCA_ERR_ARGUMENT, "null state");
    if (((uintptr_t)state & 15u) != 0) return nfail(GBCA_ERR_ARGUMENT, "the state must be 16-byte aligned");
    if (pitch < desc->n1) return nfail(GBCA_ERR_ARGUMENT, "pitch %lld is below n1 = %lld", (long long)pitch,
                                       (long long)desc->n1);
    if (nsteps < 0) return nfail(GBCA_ERR_ARGUMENT, "nsteps must be non-negative, got %lld", (long long)nsteps);
    const double need = (double)pitch * (double)desc->n2;
    if (need > (double)GBCA_NOALLOC_SCRATCH_BYTES)
        return nfail(GBCA_ERR_ARGUMENT,
                     "the state needs %.0f bytes of scratch (pitch %lld x %lld columns); gbca_advance_noalloc holds "
                     "%d bytes",
                     need, (long long)pitch, (long long)desc->n2, GBCA_NOALLOC_SCRATCH_BYTES);
    if (desc->rule == GBCA_RULE_FOREST_FIRE && (!params || nparams < 2))
        return nfail(GBCA_ERR_ARGUMENT, "the forest-fire rule needs parameters (p, f)");
    if (nsteps == 0) return GBCA_OK;
    void* scratch = nullptr;
    cudaError_t e = scratch_address(&scratch);
    if (e != cudaSuccess) return nfail(GBCA_ERR_CUDA, "scratch address: %s", cudaGetErrorString(e));
    cudaStream_t st = (cudaStream_t)stream;

    SweepParams p;
    std::memset(&p, 0, sizeof p);
    p.n1 = desc->n1;
    p.n2 = desc->n2;
    p.pitch = pitch;
    for (int a = 0; a < 2; ++a) {
        p.bnd[a] = desc->boundary[a];
        p.cval[a] = desc->boundary[a] == GBCA_CONSTANT ? (int32_t)desc->constant[a] : 0;
    }
    p.rule = desc->rule;
    p.nbhd = desc->nbhd;
    p.radius = desc->radius;
    p.states = desc->states;
    p.birth = desc->birth;
    p.survive = desc->survive;
    p.seed = desc->seed;
    p.scheme = desc->scheme;
    p.gate_f32 = desc->scheme_p_f32;
    p.gate_thr = desc->scheme == GBCA_STOCHASTIC ? gbca_threshold(desc->scheme_p, desc->scheme_p_f32) : 0;
    p.params_f32 = desc->params_f32;
    p.ngates = desc->scheme == GBCA_CHECKERBOARD ? 2 : 1;
    if (desc->rule == GBCA_RULE_FOREST_FIRE) {
        p.thr_p = gbca_threshold(params[0], desc->params_f32);
        p.thr_f = gbca_threshold(params[1], desc->params_f32);
    }
    const bool fire = fire_fast_supported(p);
    const bool life = !fire && life_simd_supported(p);
    int8_t* bufs[2] = {(int8_t*)state, (int8_t*)scratch};
    int cur = 0;
    if (fire && fire_gated(p)) {  // a gate or a mask: one sub-step per launch
        for (; nsteps > 0; ++t, --nsteps) {
            e = fire_gated_step(p, bufs, &cur, t, st);
            if (e != cudaSuccess) return nfail(GBCA_ERR_CUDA, "sweep launch: %s", cudaGetErrorString(e));
        }
    }
    while (nsteps > 0) {
        int64_t k;
        const int8_t* src = bufs[cur];
        int8_t* dst = bufs[cur ^ 1];
        p.t0 = t;
        if (fire) {
            k = nsteps < 8 ? nsteps : 8;
            p.nsub = (int32_t)k;
            e = launch_fire(p, src, dst, st);
        } else if (life) {
            const int64_t per = life_steps_per_pass(p);
            k = nsteps < per ? nsteps : per;
            p.nsub = (int32_t)(k * p.ngates);  // sub-steps: two half-steps per Checkerboard step
            e = launch_life_simd(p, src, dst, st);
        } else {
            int64_t per = kGenericSubsteps / (p.radius * p.ngates);
            if (per < 1) per = 1;
            k = nsteps < per ? nsteps : per;
            p.nsub = (int32_t)(k * p.ngates);
            p.tile_x = p.tile_y = 64;
            p.halo_x = p.halo_y = p.nsub * p.radius;
            e = launch_generic(p, src, dst, st);
        }
        if (e != cudaSuccess) return nfail(GBCA_ERR_CUDA, "sweep launch: %s", cudaGetErrorString(e));
        count_launch();
        cur ^= 1;
        t += k;
        nsteps -= k;
    }
    if (cur == 1) {  // the result is in the scratch array: copy it back into the caller's state
        e = cudaMemcpy2DAsync(state, (size_t)pitch, scratch, (size_t)pitch, (size_t)desc->n1, (size_t)desc->n2,
                              cudaMemcpyDeviceToDevice, st);
        if (e != cudaSuccess) return nfail(GBCA_ERR_CUDA, "copy back: %s", cudaGetErrorString(e));
    }
    return GBCA_OK;
}
