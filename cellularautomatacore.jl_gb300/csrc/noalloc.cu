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
// cudaGetSymbolAddress, with that device current, and caches it under the identity of the
// current CUDA context (cuCtxGetId), so a context that was destroyed and created again (after
// cudaDeviceReset, say, when the module reloads and the array may move) gets a fresh lookup
// rather than a stale address. That first call should come before any stream capture on the
// device.
//
// The sweep itself is the one gbca_advance runs (sweep_int8: the same kernels, tuned or
// pinned geometry and TMA staging), between the caller's state and the array, so results
// are gbca_advance's bit for bit. The states are not scanned first (that would need a device
// flag of its own): Generations, and Life under a gate or a mask, run the general kernel,
// which reads any state; the forest fire compares whole bytes on its first step only.
#include <cmath>
#include <cstdarg>
#include <cstdio>
#include <cstring>
#include <mutex>

#include <cuda.h>

#include "gbca_internal.cuh"

namespace gbca {

namespace {

static __device__ __align__(256) int8_t g_noalloc_scratch[GBCA_NOALLOC_SCRATCH_BYTES];

// Looked-up addresses by (device, context id): a handful of contexts per process at most.
constexpr int kMaxContexts = 64;
struct ScratchEntry {
    int dev;
    unsigned long long ctx_id;
    void* addr;
};
std::mutex g_scratch_mutex;
ScratchEntry g_scratch[kMaxContexts];
int g_scratch_n = 0;

typedef CUresult (*CtxGetCurrent)(CUcontext*);
typedef CUresult (*CtxGetId)(CUcontext, unsigned long long*);
CtxGetCurrent g_ctx_current = nullptr;
CtxGetId g_ctx_id = nullptr;
bool g_ctx_looked = false;

// The id of the calling thread's current context, or false when there is none yet (the
// runtime creates the device's primary context on its first call that needs one).
bool current_context_id(unsigned long long* id) {
    if (!g_ctx_looked) {
        g_ctx_looked = true;
        void* fn = nullptr;
        cudaDriverEntryPointQueryResult q;
        if (cudaGetDriverEntryPointByVersion("cuCtxGetCurrent", &fn, 12000, cudaEnableDefault, &q) == cudaSuccess &&
            q == cudaDriverEntryPointSuccess)
            g_ctx_current = (CtxGetCurrent)fn;
        if (cudaGetDriverEntryPointByVersion("cuCtxGetId", &fn, 12000, cudaEnableDefault, &q) == cudaSuccess &&
            q == cudaDriverEntryPointSuccess)
            g_ctx_id = (CtxGetId)fn;
        cudaGetLastError();
    }
    CUcontext ctx = nullptr;
    if (!g_ctx_current || !g_ctx_id || g_ctx_current(&ctx) != CUDA_SUCCESS || !ctx) return false;
    return g_ctx_id(ctx, id) == CUDA_SUCCESS;
}

int nfail(int code, const char* fmt, ...) {
    char msg[512];
    va_list ap;
    va_start(ap, fmt);
    vsnprintf(msg, sizeof msg, fmt, ap);
    va_end(ap);
    set_last_error(msg);
    return code;
}

// The device address of the scratch array in the current context of the current device
// (looked up once per context).
cudaError_t scratch_address(void** out) {
    int dev = 0;
    cudaError_t e = cudaGetDevice(&dev);
    if (e != cudaSuccess) return e;
    std::lock_guard<std::mutex> lock(g_scratch_mutex);
    unsigned long long id = 0;
    const bool have_id = current_context_id(&id);
    if (have_id)
        for (int i = 0; i < g_scratch_n; ++i)
            if (g_scratch[i].dev == dev && g_scratch[i].ctx_id == id) {
                *out = g_scratch[i].addr;
                return cudaSuccess;
            }
    void* p = nullptr;
    e = cudaGetSymbolAddress(&p, g_noalloc_scratch);  // creates the primary context if needed
    if (e != cudaSuccess) return e;
    if (have_id || current_context_id(&id)) {
        ScratchEntry& slot = g_scratch[g_scratch_n < kMaxContexts ? g_scratch_n++ : (int)(id % kMaxContexts)];
        slot = ScratchEntry{dev, id, p};
    }
    *out = p;
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
    int8_t* bufs[2] = {(int8_t*)state, (int8_t*)scratch};
    int cur = 0;
    e = sweep_int8(*desc, pitch, bufs, &cur, t, nsteps, params, st);
    if (e != cudaSuccess) return nfail(GBCA_ERR_CUDA, "sweep launch: %s", cudaGetErrorString(e));
    if (cur == 1) {  // the result is in the scratch array: copy it back into the caller's state
        e = cudaMemcpy2DAsync(state, (size_t)pitch, scratch, (size_t)pitch, (size_t)desc->n1, (size_t)desc->n2,
                              cudaMemcpyDeviceToDevice, st);
        if (e != cudaSuccess) return nfail(GBCA_ERR_CUDA, "copy back: %s", cudaGetErrorString(e));
    }
    return GBCA_OK;
}
