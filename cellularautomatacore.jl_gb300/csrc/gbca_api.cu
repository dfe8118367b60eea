// gbca_api.cu — the C ABI of libgbca.so (include/gbca.h): handles, state transfer,
// advance with kernel selection, single-cell access and device summaries.
#include <algorithm>
#include <cmath>
#include <cstdarg>
#include <cstdio>
#include <cstring>
#include <string>
#include <vector>

#include "field.cuh"
#include "gbca_internal.cuh"
#include "lenia.cuh"
#include "measures.cuh"

struct gbca_handle {
    gbca_desc d;
    size_t esize = 1;
    int64_t pitch = 0;  // bytes between columns
    void* buf[2] = {nullptr, nullptr};
    int cur = 0;
    cudaStream_t stream = nullptr;      // the stream work is queued on
    cudaStream_t own_stream = nullptr;  // the handle's own stream
    unsigned long long* acc = nullptr;       // device accumulator for summaries
    unsigned long long* acc_host = nullptr;  // pinned copy
    int nsm = 148;
    gbca::LeniaPlan* lenia = nullptr;
    bool states_valid = true;  // every state is one the rule produces (see scan_states)
    bool forced = false;       // gbca_set_geometry pinned the sweep geometry
    gbca::SweepChoice force = {0, 0, 0};
    // the environment (gbca_set_mask / gbca_set_field / gbca_set_covariate)
    uint8_t* mask = nullptr;           // pitch bytes between columns
    int2* taps = nullptr;
    double* w64 = nullptr;
    float* w32 = nullptr;
    int32_t ntaps = 0, field_R = 0, field_f32 = 0, field_source = 0;
    gbca::FieldFFT* field_fft = nullptr;
    void* cov = nullptr;
    int64_t cov_nt = 0;
    int32_t cov_f32 = 0;
    // saved states staged on the device and copied out on a second stream (gbca_snapshot)
    struct Snapshot {
        void* dev = nullptr;          // packed n1 x n2 copy of the state
        void* host = nullptr;         // pinned host copy
        cudaEvent_t staged = nullptr;  // the device copy is complete
        cudaEvent_t done = nullptr;    // the host copy is complete
        int64_t ticket = 0;
        bool busy = false;
    };
    std::vector<Snapshot> snaps;
    cudaStream_t copy_stream = nullptr;
    int64_t next_ticket = 1;
    // active-tile scheduling (gbca_set_sparse)
    bool sparse_on = false;
    bool sparse_dirty = true;  // the state changed outside a sweep: flags and buffers to rebuild
    gbca::SparseTiles sparse = {};
    // the lattice as a slab of a larger one (gbca_set_slab)
    bool slab_on = false;
    gbca::SlabPlace slab = {0, 0};
};

namespace {

thread_local std::string g_err;

int fail(int code, const char* fmt, ...) {
    char msg[512];
    va_list ap;
    va_start(ap, fmt);
    vsnprintf(msg, sizeof msg, fmt, ap);
    va_end(ap);
    g_err = msg;
    return code;
}

int cuda_fail(cudaError_t e, const char* what) {
    return fail(GBCA_ERR_CUDA, "%s: %s", what, cudaGetErrorString(e));
}

// A tile-copy wait that gave up leaves its tile unwritten: report it once the work is done.
int check_timeouts() {
    const int n = gbca::fire_tma_timeouts_take();
    if (n) return fail(GBCA_ERR_TIMEOUT, "%d tile copies did not complete within their wait limit", n);
    return GBCA_OK;
}

#define GBCA_CUDA(call, what)                          \
    do {                                               \
        cudaError_t e_ = (call);                       \
        if (e_ != cudaSuccess) return cuda_fail(e_, what); \
    } while (0)

bool is_int8_rule(int32_t r) {
    return r == GBCA_RULE_LIFE || r == GBCA_RULE_GENERATIONS || r == GBCA_RULE_FOREST_FIRE || r == GBCA_RULE_SI_FIELD;
}

int check_desc(const gbca_desc* d) {
    if (!d) return fail(GBCA_ERR_ARGUMENT, "null problem description");
    if (d->rule < GBCA_RULE_LIFE || d->rule > GBCA_RULE_SI_FIELD)
        return fail(GBCA_ERR_ARGUMENT,
                    "GB300Backend runs Life, Generations, forest-fire, kernel-field SI and Lenia rules; got rule kind %d",
                    d->rule);
    if (d->n1 <= 0 || d->n2 <= 0)
        return fail(GBCA_ERR_ARGUMENT, "lattice dimensions must be positive, got (%lld, %lld)", (long long)d->n1,
                    (long long)d->n2);
    if (d->n1 > (int64_t)1 << 31 || d->n2 > (int64_t)1 << 31 || d->n1 * d->n2 > ((int64_t)1 << 40))
        return fail(GBCA_ERR_ARGUMENT, "lattice of %lld x %lld cells is too large", (long long)d->n1,
                    (long long)d->n2);
    for (int a = 0; a < 2; ++a)
        if (d->boundary[a] < GBCA_PERIODIC || d->boundary[a] > GBCA_CONSTANT)
            return fail(GBCA_ERR_ARGUMENT, "unknown boundary kind %d on axis %d", d->boundary[a], a + 1);
    if (d->scheme < GBCA_SYNCHRONOUS || d->scheme > GBCA_CHECKERBOARD)
        return fail(GBCA_ERR_UNSUPPORTED, "GB300Backend runs Synchronous, Stochastic and Checkerboard schemes");
    if (d->scheme == GBCA_STOCHASTIC && !(d->scheme_p > 0.0 && d->scheme_p <= 1.0))
        return fail(GBCA_ERR_ARGUMENT, "update probability must be in (0, 1], got %g", d->scheme_p);
    if (is_int8_rule(d->rule)) {
        if (d->nbhd != GBCA_MOORE && d->nbhd != GBCA_VON_NEUMANN)
            return fail(GBCA_ERR_ARGUMENT, "GB300Backend runs Moore(r) and VonNeumann(r) neighbourhoods");
        if (d->radius < 1 || d->radius > 64)
            return fail(GBCA_ERR_ARGUMENT, "neighbourhood radius must be in 1:64, got %d", d->radius);
        for (int a = 0; a < 2; ++a) {
            if (d->boundary[a] != GBCA_CONSTANT) continue;
            const double v = d->constant[a];
            if (!(v == std::floor(v) && v >= -128.0 && v <= 127.0))
                return fail(GBCA_ERR_INCOMPATIBLE_SPACE,
                            "the boundary Constant(%g) does not fit: a state of Int8 cannot hold it", v);
        }
        if (d->rule == GBCA_RULE_GENERATIONS && (d->states < 2 || d->states > 127))
            return fail(GBCA_ERR_ARGUMENT, "a Generations rule needs 2 to 127 states on Int8, got %d", d->states);
    } else {
        if (d->lenia_R < 1 || d->lenia_R > 64)
            return fail(GBCA_ERR_ARGUMENT, "Lenia radius R must be in 1:64, got %d", d->lenia_R);
        if (d->lenia_npeaks < 1 || d->lenia_npeaks > GBCA_MAX_PEAKS)
            return fail(GBCA_ERR_ARGUMENT, "Lenia needs 1 to %d peaks, got %d", GBCA_MAX_PEAKS, d->lenia_npeaks);
        if (!(d->lenia_sigma > 0.0)) return fail(GBCA_ERR_ARGUMENT, "sigma must be positive, got %g", d->lenia_sigma);
        if (!(d->lenia_dt > 0.0 && d->lenia_dt <= 1.0))
            return fail(GBCA_ERR_ARGUMENT, "dt must be in (0, 1], got %g", d->lenia_dt);
        if (d->scheme != GBCA_SYNCHRONOUS)
            return fail(GBCA_ERR_UNSUPPORTED, "GB300Backend runs Lenia with Synchronous() only");
        if (d->lenia_method == GBCA_FFT && (d->boundary[0] != GBCA_PERIODIC || d->boundary[1] != GBCA_PERIODIC))
            return fail(GBCA_ERR_ARGUMENT,
                        "field :potential uses method=:fft, which needs periodic boundaries on every axis");
        for (int a = 0; a < 2; ++a)
            if (d->boundary[a] == GBCA_CONSTANT && d->constant[a] != 0.0)
                return fail(GBCA_ERR_UNSUPPORTED, "GB300Backend runs Lenia with Constant(0) edges only");
    }
    return GBCA_OK;
}

uint64_t threshold(double p, bool f32) {
    if (f32) {
        const float pf = (float)p;
        if (!(pf > 0.0f)) return 0;
        if (pf >= 1.0f) return (uint64_t)1 << 24;
        return (uint64_t)std::ceil((double)pf * 16777216.0);
    }
    if (!(p > 0.0)) return 0;
    if (p >= 1.0) return (uint64_t)1 << 53;
    return (uint64_t)std::ceil(p * 9007199254740992.0);
}

// Whether every cell of the current state is one the rule produces — 0..C-1 for Generations,
// 0..2 for the forest fire, 0..1 for gated Life — by one byte-compare pass over the state
// (an HBM-speed read), or from a device histogram where the buffer layout does not allow it.
cudaError_t scan_states(gbca_handle* h, bool* valid) {
    const int nv = h->d.rule == GBCA_RULE_GENERATIONS ? h->d.states : (h->d.rule == GBCA_RULE_LIFE ? 2 : 3);
    const int8_t* u = (const int8_t*)h->buf[h->cur];
    if (h->pitch % 16 == 0 && ((uintptr_t)u & 15u) == 0) {
        unsigned int* bad = (unsigned int*)h->acc;
        cudaError_t e = gbca::launch_states_in_range(u, h->d.n1, h->d.n2, h->pitch, nv, bad, h->nsm, h->stream);
        if (e == cudaSuccess)
            e = cudaMemcpyAsync(h->acc_host, bad, sizeof(unsigned int), cudaMemcpyDeviceToHost, h->stream);
        if (e == cudaSuccess) e = cudaStreamSynchronize(h->stream);
        if (e != cudaSuccess) return e;
        *valid = *(const unsigned int*)h->acc_host == 0u;
        return cudaSuccess;
    }
    cudaError_t e = gbca::launch_measures(u, h->d.n1, h->d.n2, h->pitch, h->d.boundary[0], h->d.boundary[1], h->acc,
                                          h->nsm, h->stream);
    if (e == cudaSuccess)
        e = cudaMemcpyAsync(h->acc_host, h->acc, 256 * sizeof(unsigned long long), cudaMemcpyDeviceToHost, h->stream);
    if (e == cudaSuccess) e = cudaStreamSynchronize(h->stream);
    if (e != cudaSuccess) return e;
    unsigned long long inside = 0;
    for (int v = 0; v < nv && v < 128; ++v) inside += h->acc_host[128 + v];
    *valid = inside == (unsigned long long)(h->d.n1 * h->d.n2);
    return cudaSuccess;
}

bool scanned_rule(const gbca_handle* h) {
    // gated or masked Life keeps closed cells' values, which its bit-sliced kernel holds only for 0 and 1
    return h->d.rule == GBCA_RULE_GENERATIONS || h->d.rule == GBCA_RULE_FOREST_FIRE ||
           (h->d.rule == GBCA_RULE_LIFE && (h->d.scheme != GBCA_SYNCHRONOUS || h->mask));
}

// A state written by the caller may hold values the rule never produces; the fast paths
// assume it does not, so scan it once (the rule keeps valid states valid).
int ensure_scanned(gbca_handle* h) {
    if (!scanned_rule(h) || h->states_valid) return GBCA_OK;
    bool valid = false;
    const cudaError_t e = scan_states(h, &valid);
    if (e != cudaSuccess) return cuda_fail(e, "state scan");
    h->states_valid = valid;
    return GBCA_OK;
}

int advance_si(gbca_handle* h, int64_t t, int64_t nsteps, const double* params, int32_t nparams) {
    if (!params || nparams < 1) return fail(GBCA_ERR_ARGUMENT, "the kernel-field SI rule needs its parameter beta");
    if (h->ntaps < 1) return fail(GBCA_ERR_ARGUMENT, "the kernel-field SI rule needs a field (gbca_set_field)");
    gbca::FieldSweep p;
    std::memset(&p, 0, sizeof p);
    p.n1 = h->d.n1;
    p.n2 = h->d.n2;
    p.pitch = h->pitch;
    for (int a = 0; a < 2; ++a) {
        p.bnd[a] = h->d.boundary[a];
        p.cval[a] = h->d.boundary[a] == GBCA_CONSTANT ? (int32_t)h->d.constant[a] : 0;
    }
    p.seed = h->d.seed;
    p.scheme = h->d.scheme;
    p.gate_f32 = h->d.scheme_p_f32;
    p.gate_thr = h->d.scheme == GBCA_STOCHASTIC ? threshold(h->d.scheme_p, h->d.scheme_p_f32 != 0) : 0;
    p.mask = h->mask;
    p.taps = h->taps;
    p.w64 = h->w64;
    p.w32 = h->w32;
    p.ntaps = h->ntaps;
    p.R = h->field_R;
    p.field_f32 = h->field_f32;
    p.source = h->field_source;
    p.cov = h->cov;
    p.cov_nt = h->cov_nt;
    p.cov_f32 = h->cov_f32;
    p.beta_f32 = h->d.params_f32;
    p.beta = h->d.params_f32 ? (double)(float)params[0] : params[0];
    int8_t* const bufs[2] = {(int8_t*)h->buf[0], (int8_t*)h->buf[1]};
    const cudaError_t e = gbca::sweep_si(p, h->field_fft, bufs, &h->cur, t, nsteps, h->nsm, h->stream);
    if (e != cudaSuccess) return cuda_fail(e, "kernel-field sweep");
    return GBCA_OK;
}

int advance_int8(gbca_handle* h, int64_t t, int64_t nsteps, const double* params, int32_t nparams) {
    if (h->d.rule == GBCA_RULE_SI_FIELD) return advance_si(h, t, nsteps, params, nparams);
    if (h->d.rule == GBCA_RULE_FOREST_FIRE && (!params || nparams < 2))
        return fail(GBCA_ERR_ARGUMENT, "the forest-fire rule needs parameters (p, f)");
    const int rc = ensure_scanned(h);
    if (rc != GBCA_OK) return rc;
    int8_t* const bufs[2] = {(int8_t*)h->buf[0], (int8_t*)h->buf[1]};
    if (h->sparse_on) {
        if (!gbca::rule_quiescent(h->d, params, h->sparse.background))
            return fail(GBCA_ERR_ARGUMENT,
                        "active-tile sweeps need a quiescent rule: a background cell (%d) with background neighbours "
                        "changes under these parameters", (int)h->sparse.background);
        if (h->sparse_dirty) {  // flags of the current state; the other buffer made equal to it
            const size_t bytes = (size_t)h->pitch * (size_t)h->d.n2;
            cudaError_t e = gbca::launch_tile_flags(bufs[h->cur], h->d.n1, h->d.n2, h->pitch, h->sparse,
                                                    h->sparse.flags[h->cur], h->stream);
            if (e == cudaSuccess)
                e = cudaMemcpyAsync(bufs[h->cur ^ 1], bufs[h->cur], bytes, cudaMemcpyDeviceToDevice, h->stream);
            if (e == cudaSuccess)
                e = cudaMemcpyAsync(h->sparse.flags[h->cur ^ 1], h->sparse.flags[h->cur],
                                    (size_t)h->sparse.tiles_x * h->sparse.tiles_y, cudaMemcpyDeviceToDevice, h->stream);
            if (e != cudaSuccess) return cuda_fail(e, "active-tile set-up");
            h->sparse_dirty = false;
        }
    }
    const cudaError_t e = gbca::sweep_int8(h->d, h->pitch, bufs, &h->cur, t, nsteps, params, h->stream,
                                           scanned_rule(h) && h->states_valid, h->forced ? &h->force : nullptr,
                                           h->mask, h->sparse_on ? &h->sparse : nullptr,
                                           h->slab_on ? &h->slab : nullptr);
    // a synchronous, unmasked step leaves only 0, 1 and 2; a closed or masked cell keeps its value
    if (h->d.rule == GBCA_RULE_FOREST_FIRE && h->d.scheme == GBCA_SYNCHRONOUS && !h->mask) h->states_valid = true;
    if (e != cudaSuccess) return cuda_fail(e, "sweep launch");
    return GBCA_OK;
}

// The sweep parameters of the handle's next call, for the kernel-selection predicates.
gbca::SweepParams handle_params(const gbca_handle* h, const double* params) {
    gbca::SweepParams p = gbca::sweep_params(h->d, h->pitch, params);
    p.states_valid = scanned_rule(h) && h->states_valid ? 1 : 0;
    p.mask = h->mask;
    if (h->slab_on) {
        p.col0 = h->slab.col0;
        p.n2g = h->slab.n2g;
    }
    return p;
}

// Times nsteps steps of each candidate geometry from the handle's current state (restored
// before every run and at the end) and returns the fastest per step.
int time_candidates(gbca_handle* h, const std::vector<gbca::SweepChoice>& cands, const double* params,
                    gbca::SweepChoice* best) {
    const size_t bytes = (size_t)h->pitch * (size_t)h->d.n2;
    const int cur0 = h->cur;
    void* saved = nullptr;
    cudaEvent_t ev[2] = {nullptr, nullptr};
    cudaError_t e = cudaMalloc(&saved, bytes);
    if (e == cudaSuccess) e = cudaMemcpyAsync(saved, h->buf[cur0], bytes, cudaMemcpyDeviceToDevice, h->stream);
    if (e == cudaSuccess) e = cudaEventCreate(&ev[0]);
    if (e == cudaSuccess) e = cudaEventCreate(&ev[1]);
    float best_ms = 0.0f;
    int8_t* const bufs[2] = {(int8_t*)h->buf[0], (int8_t*)h->buf[1]};
    const bool valid = scanned_rule(h) && h->states_valid;
    for (size_t c = 0; c < cands.size() && e == cudaSuccess; ++c) {
        // a whole number of passes, about 48 steps, so that every candidate runs full passes
        const int per = cands[c].steps_per_pass;
        const int64_t nsteps = (int64_t)per * ((48 + per - 1) / per);
        float ms_min = 0.0f;
        for (int rep = 0; rep < 3 && e == cudaSuccess; ++rep) {
            h->cur = cur0;
            e = cudaMemcpyAsync(h->buf[cur0], saved, bytes, cudaMemcpyDeviceToDevice, h->stream);
            if (e == cudaSuccess) e = cudaEventRecord(ev[0], h->stream);
            if (e == cudaSuccess)
                e = gbca::sweep_int8(h->d, h->pitch, bufs, &h->cur, 1, nsteps, params, h->stream, valid, &cands[c],
                                     h->mask, nullptr, h->slab_on ? &h->slab : nullptr);
            if (e == cudaSuccess) e = cudaEventRecord(ev[1], h->stream);
            if (e == cudaSuccess) e = cudaEventSynchronize(ev[1]);
            float ms = 0.0f;
            if (e == cudaSuccess) e = cudaEventElapsedTime(&ms, ev[0], ev[1]);
            ms /= (float)nsteps;
            if (rep == 0 || ms < ms_min) ms_min = ms;
        }
        if (e == cudaSuccess && (c == 0 || ms_min < best_ms)) {
            best_ms = ms_min;
            *best = cands[c];
        }
    }
    h->cur = cur0;
    h->sparse_dirty = true;  // the other buffer now holds a candidate's result
    if (saved) {
        const cudaError_t e2 = cudaMemcpyAsync(h->buf[cur0], saved, bytes, cudaMemcpyDeviceToDevice, h->stream);
        if (e == cudaSuccess) e = e2;
        const cudaError_t e3 = cudaStreamSynchronize(h->stream);
        if (e == cudaSuccess) e = e3;
        cudaFree(saved);
    }
    for (cudaEvent_t x : ev)
        if (x) cudaEventDestroy(x);
    if (e != cudaSuccess) {
        cudaGetLastError();
        return e == cudaErrorMemoryAllocation ? fail(GBCA_ERR_OUT_OF_MEMORY, "the tuner's copy of the state (%zu bytes) "
                                                     "did not fit", bytes)
                                              : cuda_fail(e, "gbca_tune");
    }
    return GBCA_OK;
}

}  // namespace

namespace gbca {
// Lets other translation units of the library report through gbca_last_error().
void set_last_error(const char* msg) { g_err = msg; }
}  // namespace gbca

extern "C" {

const char* gbca_last_error(void) { return g_err.c_str(); }

int32_t gbca_version(void) { return 100; }

int32_t gbca_device_count(void) {
    int n = 0;
    if (cudaGetDeviceCount(&n) != cudaSuccess) {
        cudaGetLastError();
        return 0;
    }
    return n;
}

uint64_t gbca_threshold(double p, int32_t f32) { return threshold(p, f32 != 0); }

int gbca_check(const gbca_desc* desc) { return check_desc(desc); }

int gbca_create(const gbca_desc* desc, gbca_handle** out) {
    if (!out) return fail(GBCA_ERR_ARGUMENT, "null output handle");
    *out = nullptr;
    int rc = check_desc(desc);
    if (rc != GBCA_OK) return rc;
    if (gbca_device_count() < 1) return fail(GBCA_ERR_CUDA, "no CUDA device is visible");
    gbca_handle* h = new gbca_handle();
    h->d = *desc;
    h->esize = desc->rule == GBCA_RULE_LENIA ? (desc->lenia_f64 ? 8 : 4) : 1;
    const int64_t row = desc->n1 * (int64_t)h->esize;
    h->pitch = (row + 127) / 128 * 128;
    int dev = 0;
    cudaGetDevice(&dev);
    cudaDeviceGetAttribute(&h->nsm, cudaDevAttrMultiProcessorCount, dev);
    const size_t bytes = (size_t)h->pitch * (size_t)desc->n2;
    cudaError_t e = cudaStreamCreateWithFlags(&h->own_stream, cudaStreamNonBlocking);
    h->stream = h->own_stream;
    if (e == cudaSuccess) e = cudaMalloc(&h->buf[0], bytes);
    if (e == cudaSuccess) e = cudaMalloc(&h->buf[1], bytes);
    if (e == cudaSuccess) e = cudaMalloc(&h->acc, gbca::kMeasureWords * sizeof(unsigned long long));
    if (e == cudaSuccess) e = cudaMallocHost(&h->acc_host, gbca::kMeasureWords * sizeof(unsigned long long));
    if (e == cudaSuccess) e = cudaMemsetAsync(h->buf[0], 0, bytes, h->stream);
    if (e == cudaSuccess) e = cudaMemsetAsync(h->buf[1], 0, bytes, h->stream);
    if (e == cudaSuccess && desc->rule == GBCA_RULE_LENIA) {
        rc = gbca::lenia_create(*desc, h->pitch, h->stream, &h->lenia, g_err);
        if (rc != GBCA_OK) {
            gbca_destroy(h);
            return rc;
        }
    }
    if (e == cudaSuccess) e = cudaStreamSynchronize(h->stream);
    if (e != cudaSuccess) {
        const bool oom = e == cudaErrorMemoryAllocation;
        gbca_destroy(h);
        cudaGetLastError();
        return oom ? fail(GBCA_ERR_OUT_OF_MEMORY, "device allocation of %zu bytes failed", 2 * bytes)
                   : cuda_fail(e, "gbca_create");
    }
    *out = h;
    return GBCA_OK;
}

int gbca_destroy(gbca_handle* h) {
    if (!h) return GBCA_OK;
    if (h->stream) cudaStreamSynchronize(h->stream);
    if (h->lenia) gbca::lenia_destroy(h->lenia);
    cudaFree(h->buf[0]);
    cudaFree(h->buf[1]);
    cudaFree(h->acc);
    cudaFree(h->mask);
    cudaFree(h->taps);
    cudaFree(h->w64);
    cudaFree(h->w32);
    cudaFree(h->cov);
    gbca::field_fft_destroy(h->field_fft);
    if (h->copy_stream) cudaStreamSynchronize(h->copy_stream);
    for (auto& sn : h->snaps) {
        cudaFree(sn.dev);
        if (sn.host) cudaFreeHost(sn.host);
        if (sn.staged) cudaEventDestroy(sn.staged);
        if (sn.done) cudaEventDestroy(sn.done);
    }
    if (h->copy_stream) cudaStreamDestroy(h->copy_stream);
    cudaFree(h->sparse.flags[0]);
    cudaFree(h->sparse.flags[1]);
    cudaFree(h->sparse.list);
    cudaFree(h->sparse.count);
    if (h->acc_host) cudaFreeHost(h->acc_host);
    if (h->own_stream) cudaStreamDestroy(h->own_stream);
    delete h;
    return GBCA_OK;
}

int gbca_set_state(gbca_handle* h, const void* host, size_t nbytes) {
    if (!h || !host) return fail(GBCA_ERR_ARGUMENT, "null handle or state");
    const size_t row = (size_t)h->d.n1 * h->esize;
    if (nbytes != row * (size_t)h->d.n2)
        return fail(GBCA_ERR_STATE, "the state has %zu bytes, the lattice needs %zu", nbytes, row * (size_t)h->d.n2);
    GBCA_CUDA(cudaMemcpy2DAsync(h->buf[h->cur], (size_t)h->pitch, host, row, row, (size_t)h->d.n2,
                                cudaMemcpyHostToDevice, h->stream),
              "set_state copy");
    h->states_valid = false;
    h->sparse_dirty = true;
    GBCA_CUDA(cudaStreamSynchronize(h->stream), "set_state");
    return GBCA_OK;
}

int gbca_set_state_async(gbca_handle* h, const void* host, size_t nbytes) {
    if (!h || !host) return fail(GBCA_ERR_ARGUMENT, "null handle or state");
    const size_t row = (size_t)h->d.n1 * h->esize;
    if (nbytes != row * (size_t)h->d.n2)
        return fail(GBCA_ERR_STATE, "the state has %zu bytes, the lattice needs %zu", nbytes, row * (size_t)h->d.n2);
    GBCA_CUDA(cudaMemcpy2DAsync(h->buf[h->cur], (size_t)h->pitch, host, row, row, (size_t)h->d.n2,
                                cudaMemcpyHostToDevice, h->stream),
              "set_state_async copy");
    h->states_valid = false;
    h->sparse_dirty = true;
    return GBCA_OK;
}

int gbca_get_state_async(gbca_handle* h, void* host, size_t nbytes) {
    if (!h || !host) return fail(GBCA_ERR_ARGUMENT, "null handle or state");
    const size_t row = (size_t)h->d.n1 * h->esize;
    if (nbytes != row * (size_t)h->d.n2)
        return fail(GBCA_ERR_STATE, "the buffer has %zu bytes, the lattice needs %zu", nbytes, row * (size_t)h->d.n2);
    GBCA_CUDA(cudaMemcpy2DAsync(host, row, h->buf[h->cur], (size_t)h->pitch, row, (size_t)h->d.n2,
                                cudaMemcpyDeviceToHost, h->stream),
              "get_state_async copy");
    return GBCA_OK;
}

int gbca_set_state_device(gbca_handle* h, const void* dptr, int64_t src_pitch) {
    if (!h || !dptr) return fail(GBCA_ERR_ARGUMENT, "null handle or state");
    const size_t row = (size_t)h->d.n1 * h->esize;
    if (src_pitch < (int64_t)row) return fail(GBCA_ERR_ARGUMENT, "source pitch %lld is below a column's %zu bytes",
                                              (long long)src_pitch, row);
    GBCA_CUDA(cudaMemcpy2DAsync(h->buf[h->cur], (size_t)h->pitch, dptr, (size_t)src_pitch, row, (size_t)h->d.n2,
                                cudaMemcpyDeviceToDevice, h->stream),
              "set_state_device copy");
    h->states_valid = false;
    h->sparse_dirty = true;
    return GBCA_OK;
}

int gbca_selftest_wait(int32_t polls) {
    if (polls < 1 || polls > (1 << 20)) return fail(GBCA_ERR_ARGUMENT, "polls must lie in 1..2^20, got %d", (int)polls);
    GBCA_CUDA(gbca::launch_wait_probe(polls, nullptr), "wait probe");
    GBCA_CUDA(cudaDeviceSynchronize(), "wait probe");
    return check_timeouts();
}

int gbca_set_state_soup(gbca_handle* h, double density, uint64_t seed) {
    if (!h) return fail(GBCA_ERR_ARGUMENT, "null handle");
    if (h->esize != 1) return fail(GBCA_ERR_UNSUPPORTED, "a soup is an Int8 state");
    if (!(density >= 0.0 && density <= 1.0)) return fail(GBCA_ERR_ARGUMENT, "density must be in [0, 1]");
    GBCA_CUDA(gbca::launch_soup((int8_t*)h->buf[h->cur], h->d.n1, h->d.n2, h->pitch, density, seed, h->nsm * 8,
                                h->stream),
              "set_state_soup");
    h->states_valid = false;
    h->sparse_dirty = true;
    return GBCA_OK;
}

int gbca_get_state(gbca_handle* h, void* host, size_t nbytes) {
    if (!h || !host) return fail(GBCA_ERR_ARGUMENT, "null handle or state");
    const size_t row = (size_t)h->d.n1 * h->esize;
    if (nbytes != row * (size_t)h->d.n2)
        return fail(GBCA_ERR_STATE, "the buffer has %zu bytes, the lattice needs %zu", nbytes, row * (size_t)h->d.n2);
    GBCA_CUDA(cudaMemcpy2DAsync(host, row, h->buf[h->cur], (size_t)h->pitch, row, (size_t)h->d.n2,
                                cudaMemcpyDeviceToHost, h->stream),
              "current_state copy");
    GBCA_CUDA(cudaStreamSynchronize(h->stream), "current_state");
    return check_timeouts();
}

int gbca_advance(gbca_handle* h, int64_t t, int64_t nsteps, const double* params, int32_t nparams) {
    if (!h) return fail(GBCA_ERR_ARGUMENT, "null handle");
    if (nsteps < 0) return fail(GBCA_ERR_ARGUMENT, "nsteps must be non-negative, got %lld", (long long)nsteps);
    if (nsteps == 0) return GBCA_OK;
    if (h->d.rule == GBCA_RULE_LENIA) {
        return gbca::lenia_advance(h->lenia, nsteps, h->stream, &h->cur, h->buf, g_err);
    }
    return advance_int8(h, t, nsteps, params, nparams);
}

int gbca_tune(gbca_handle* h, const double* params, int32_t nparams, int32_t* steps_per_pass, int32_t* tile_rows,
              int32_t* staging) {
    if (!h) return fail(GBCA_ERR_ARGUMENT, "null handle");
    if (steps_per_pass) *steps_per_pass = 0;
    if (tile_rows) *tile_rows = 0;
    if (staging) *staging = 0;
    if (h->d.rule == GBCA_RULE_LENIA || h->d.rule == GBCA_RULE_SI_FIELD) return GBCA_OK;  // nothing to tune
    if (h->d.rule == GBCA_RULE_FOREST_FIRE && (!params || nparams < 2))
        return fail(GBCA_ERR_ARGUMENT, "the forest-fire rule needs parameters (p, f)");
    int rc = ensure_scanned(h);
    if (rc != GBCA_OK) return rc;
    const std::vector<gbca::SweepChoice> cands = gbca::sweep_candidates(handle_params(h, params));
    if (cands.empty()) return GBCA_OK;  // the general kernel: one geometry
    gbca::SweepChoice best = cands[0];
    rc = time_candidates(h, cands, params, &best);
    if (rc != GBCA_OK) return rc;
    gbca::store_choice(h->d, best);
    if (steps_per_pass) *steps_per_pass = best.steps_per_pass;
    if (tile_rows) *tile_rows = best.tile_rows;
    if (staging) *staging = best.staging;
    return GBCA_OK;
}

int gbca_geometry(gbca_handle* h, const double* params, int32_t* steps_per_pass, int32_t* tile_rows,
                  int32_t* staging) {
    if (!h) return fail(GBCA_ERR_ARGUMENT, "null handle");
    gbca::SweepChoice c = {0, 0, 0};
    if (h->d.rule != GBCA_RULE_LENIA && h->d.rule != GBCA_RULE_SI_FIELD && !h->sparse_on) {
        const gbca::SweepParams p = handle_params(h, params);
        const bool fire = gbca::fire_fast_supported(p), life = !fire && gbca::life_simd_supported(p);
        if (fire || life) c = gbca::sweep_choice(h->d, fire, life, h->forced ? &h->force : nullptr);
    }
    if (steps_per_pass) *steps_per_pass = c.steps_per_pass;
    if (tile_rows) *tile_rows = c.tile_rows;
    if (staging) *staging = c.staging;
    return GBCA_OK;
}

int gbca_forget_tuning(void) {
    gbca::forget_choices();
    return GBCA_OK;
}

int gbca_set_geometry(gbca_handle* h, int32_t steps_per_pass, int32_t tile_rows, int32_t staging) {
    if (!h) return fail(GBCA_ERR_ARGUMENT, "null handle");
    if (steps_per_pass == 0 && tile_rows == 0 && staging == 0) {
        h->forced = false;
        return GBCA_OK;
    }
    if (steps_per_pass < 1 || steps_per_pass > 64 || tile_rows < 0 || staging < 0 || staging > 2)
        return fail(GBCA_ERR_ARGUMENT,
                    "steps per pass must lie in 1..64, tile rows be non-negative and staging 0..2, got %d, %d, %d",
                    (int)steps_per_pass, (int)tile_rows, (int)staging);
    if (h->d.rule == GBCA_RULE_LENIA || h->d.rule == GBCA_RULE_SI_FIELD)
        return fail(GBCA_ERR_UNSUPPORTED, "sweep geometry applies to the Int8 stencil kernels only");
    const int rc = ensure_scanned(h);
    if (rc != GBCA_OK) return rc;
    const gbca::SweepParams p = handle_params(h, nullptr);
    if (gbca::fire_fast_supported(p)) {
        if (tile_rows != 0 && !gbca::fire_rows_fit(steps_per_pass, tile_rows, staging))
            return fail(GBCA_ERR_ARGUMENT,
                        "forest-fire tiles take %d..%d rows within shared memory; got %d rows at %d steps per pass",
                        gbca::kFireRowsMin, gbca::kFireRowsMax, (int)tile_rows, (int)steps_per_pass);
        // (a gated or masked fire runs one sub-step per launch whatever steps_per_pass says)
    } else if (gbca::life_simd_supported(p)) {
        if (staging != 0) return fail(GBCA_ERR_ARGUMENT, "the bit-sliced kernel stages its tiles one way; pass 0");
        if (tile_rows > 0 && !gbca::life_choice_fits(p, steps_per_pass, tile_rows))
            return fail(GBCA_ERR_ARGUMENT, "%d steps per pass on tiles %d rows high exceed shared memory",
                        (int)steps_per_pass, (int)tile_rows);
    } else {
        return fail(GBCA_ERR_UNSUPPORTED, "this problem runs on the general kernel, whose geometry is fixed");
    }
    h->force.steps_per_pass = steps_per_pass;
    h->force.tile_rows = tile_rows;
    h->force.staging = staging;
    h->forced = true;
    return GBCA_OK;
}

int gbca_set_mask(gbca_handle* h, const uint8_t* host, size_t nbytes) {
    if (!h) return fail(GBCA_ERR_ARGUMENT, "null handle");
    if (h->d.rule == GBCA_RULE_LENIA) return fail(GBCA_ERR_UNSUPPORTED, "GB300Backend runs masks with Int8 rules only");
    GBCA_CUDA(cudaStreamSynchronize(h->stream), "set_mask");
    if (!host) {
        cudaFree(h->mask);
        h->mask = nullptr;
        return GBCA_OK;
    }
    const size_t n1 = (size_t)h->d.n1, n2 = (size_t)h->d.n2;
    if (nbytes != n1 * n2) return fail(GBCA_ERR_STATE, "the mask has %zu cells, the lattice %zu", nbytes, n1 * n2);
    if (!h->mask) GBCA_CUDA(cudaMalloc(&h->mask, (size_t)h->pitch * n2), "mask allocation");
    GBCA_CUDA(cudaMemcpy2DAsync(h->mask, (size_t)h->pitch, host, n1, n1, n2, cudaMemcpyHostToDevice, h->stream),
              "mask copy");
    GBCA_CUDA(cudaStreamSynchronize(h->stream), "set_mask");
    return GBCA_OK;
}

int gbca_set_field(gbca_handle* h, int32_t ntaps, const int32_t* taps, const double* weights, int32_t f32,
                   int32_t source, int32_t method) {
    if (!h) return fail(GBCA_ERR_ARGUMENT, "null handle");
    if (h->d.rule != GBCA_RULE_SI_FIELD)
        return fail(GBCA_ERR_UNSUPPORTED, "only the kernel-field SI rule reads a kernel field");
    if (ntaps < 1 || !taps || !weights) return fail(GBCA_ERR_ARGUMENT, "a kernel field needs at least one tap");
    if (source != GBCA_SOURCE_INDICATOR && source != GBCA_SOURCE_IDENTITY)
        return fail(GBCA_ERR_ARGUMENT, "unknown field source %d", (int)source);
    if (method != GBCA_DIRECT && method != GBCA_FFT) return fail(GBCA_ERR_ARGUMENT, "method must be direct or fft");
    int R = 0;
    for (int k = 0; k < 2 * ntaps; ++k) R = std::max(R, std::abs(taps[k]));
    if (method == GBCA_DIRECT && R > 64)
        return fail(GBCA_ERR_UNSUPPORTED, "direct kernel fields reach at most 64 cells, this one %d; use method=:fft", R);
    if (method == GBCA_FFT && (h->d.boundary[0] != GBCA_PERIODIC || h->d.boundary[1] != GBCA_PERIODIC))
        return fail(GBCA_ERR_ARGUMENT, "a field with method=:fft needs periodic boundaries on every axis");
    GBCA_CUDA(cudaStreamSynchronize(h->stream), "set_field");
    cudaFree(h->taps);
    cudaFree(h->w64);
    cudaFree(h->w32);
    gbca::field_fft_destroy(h->field_fft);
    h->taps = nullptr;
    h->w64 = nullptr;
    h->w32 = nullptr;
    h->field_fft = nullptr;
    h->ntaps = 0;
    std::vector<int2> t2((size_t)ntaps);
    std::vector<float> wf((size_t)ntaps);
    for (int k = 0; k < ntaps; ++k) {
        t2[k] = make_int2(taps[2 * k], taps[2 * k + 1]);
        wf[k] = (float)weights[k];
    }
    GBCA_CUDA(cudaMalloc(&h->taps, sizeof(int2) * ntaps), "field allocation");
    GBCA_CUDA(cudaMalloc(&h->w64, sizeof(double) * ntaps), "field allocation");
    GBCA_CUDA(cudaMalloc(&h->w32, sizeof(float) * ntaps), "field allocation");
    GBCA_CUDA(cudaMemcpyAsync(h->taps, t2.data(), sizeof(int2) * ntaps, cudaMemcpyHostToDevice, h->stream), "field copy");
    GBCA_CUDA(cudaMemcpyAsync(h->w64, weights, sizeof(double) * ntaps, cudaMemcpyHostToDevice, h->stream), "field copy");
    GBCA_CUDA(cudaMemcpyAsync(h->w32, wf.data(), sizeof(float) * ntaps, cudaMemcpyHostToDevice, h->stream), "field copy");
    if (method == GBCA_FFT) {
        std::vector<int> tv(taps, taps + 2 * ntaps);
        std::vector<double> wv(weights, weights + ntaps);
        const int rc = gbca::field_fft_create(h->d.n1, h->d.n2, tv, wv, f32 != 0, h->stream, &h->field_fft, g_err);
        if (rc != GBCA_OK) return rc;
    }
    GBCA_CUDA(cudaStreamSynchronize(h->stream), "set_field");
    h->ntaps = ntaps;
    h->field_R = R;
    h->field_f32 = f32 != 0;
    h->field_source = source;
    return GBCA_OK;
}

int gbca_set_covariate(gbca_handle* h, const void* host, int64_t nt, int32_t f32) {
    if (!h) return fail(GBCA_ERR_ARGUMENT, "null handle");
    if (h->d.rule != GBCA_RULE_SI_FIELD) return fail(GBCA_ERR_UNSUPPORTED, "only the kernel-field SI rule reads a covariate");
    GBCA_CUDA(cudaStreamSynchronize(h->stream), "set_covariate");
    cudaFree(h->cov);
    h->cov = nullptr;
    h->cov_nt = 0;
    if (!host) return GBCA_OK;
    if (nt < 1) return fail(GBCA_ERR_ARGUMENT, "a covariate needs at least one time slice, got %lld", (long long)nt);
    const size_t bytes = (size_t)h->d.n1 * (size_t)h->d.n2 * (size_t)nt * (f32 ? sizeof(float) : sizeof(double));
    GBCA_CUDA(cudaMalloc(&h->cov, bytes), "covariate allocation");
    GBCA_CUDA(cudaMemcpyAsync(h->cov, host, bytes, cudaMemcpyHostToDevice, h->stream), "covariate copy");
    GBCA_CUDA(cudaStreamSynchronize(h->stream), "set_covariate");
    h->cov_nt = nt;
    h->cov_f32 = f32 != 0;
    return GBCA_OK;
}

int gbca_read_cell(gbca_handle* h, int64_t i, int64_t j, void* out) {
    if (!h || !out) return fail(GBCA_ERR_ARGUMENT, "null handle or output");
    if (i < 1 || i > h->d.n1 || j < 1 || j > h->d.n2)
        return fail(GBCA_ERR_ARGUMENT, "index (%lld, %lld) is outside the %lld x %lld lattice", (long long)i,
                    (long long)j, (long long)h->d.n1, (long long)h->d.n2);
    const char* src = (const char*)h->buf[h->cur] + (i - 1) * (int64_t)h->esize + (j - 1) * h->pitch;
    GBCA_CUDA(cudaMemcpyAsync(out, src, h->esize, cudaMemcpyDeviceToHost, h->stream), "read_cell");
    GBCA_CUDA(cudaStreamSynchronize(h->stream), "read_cell");
    return GBCA_OK;
}

int gbca_write_cell(gbca_handle* h, int64_t i, int64_t j, const void* value) {
    if (!h || !value) return fail(GBCA_ERR_ARGUMENT, "null handle or value");
    if (i < 1 || i > h->d.n1 || j < 1 || j > h->d.n2)
        return fail(GBCA_ERR_ARGUMENT, "index (%lld, %lld) is outside the %lld x %lld lattice", (long long)i,
                    (long long)j, (long long)h->d.n1, (long long)h->d.n2);
    char* dst = (char*)h->buf[h->cur] + (i - 1) * (int64_t)h->esize + (j - 1) * h->pitch;
    GBCA_CUDA(cudaMemcpyAsync(dst, value, h->esize, cudaMemcpyHostToDevice, h->stream), "write_cell");
    h->states_valid = false;
    h->sparse_dirty = true;
    GBCA_CUDA(cudaStreamSynchronize(h->stream), "write_cell");
    return GBCA_OK;
}

int gbca_sync(gbca_handle* h) {
    if (!h) return fail(GBCA_ERR_ARGUMENT, "null handle");
    GBCA_CUDA(cudaStreamSynchronize(h->stream), "sync");
    return check_timeouts();
}

int gbca_set_sparse(gbca_handle* h, int32_t enable, int32_t background, int32_t tilesize) {
    if (!h) return fail(GBCA_ERR_ARGUMENT, "null handle");
    GBCA_CUDA(cudaStreamSynchronize(h->stream), "set_sparse");
    if (!enable) {
        h->sparse_on = false;
        return GBCA_OK;
    }
    if (h->d.rule == GBCA_RULE_LENIA || h->d.rule == GBCA_RULE_SI_FIELD)
        return fail(GBCA_ERR_ARGUMENT, "active-tile sweeps run rules without kernel fields (Life, Generations, forest fire)");
    if (h->d.scheme == GBCA_CHECKERBOARD)
        return fail(GBCA_ERR_UNSUPPORTED, "active-tile sweeps run Synchronous() and Stochastic(p)");
    if (h->slab_on) return fail(GBCA_ERR_UNSUPPORTED, "a slab of a larger lattice runs dense sweeps only");
    if (background < -128 || background > 127) return fail(GBCA_ERR_ARGUMENT, "the background must be an Int8 value");
    if (tilesize <= 0) tilesize = 64;
    if (tilesize < 8 || tilesize > 128)
        return fail(GBCA_ERR_ARGUMENT, "tile side must lie in 8:128, got %d", (int)tilesize);
    if (h->d.rule != GBCA_RULE_FOREST_FIRE && !gbca::rule_quiescent(h->d, nullptr, background))
        return fail(GBCA_ERR_ARGUMENT,
                    "active-tile sweeps need a quiescent rule: a background cell (%d) with background neighbours "
                    "changes", (int)background);
    const int tile_w = (tilesize + 31) / 32 * 32;  // whole 32-cell words for the bit-sliced kernel
    const int tx = (int)((h->d.n1 + tile_w - 1) / tile_w), ty = (int)((h->d.n2 + tilesize - 1) / tilesize);
    cudaFree(h->sparse.flags[0]);
    cudaFree(h->sparse.flags[1]);
    cudaFree(h->sparse.list);
    cudaFree(h->sparse.count);
    h->sparse = {};
    const size_t n = (size_t)tx * ty;
    cudaError_t e = cudaMalloc(&h->sparse.flags[0], n);
    if (e == cudaSuccess) e = cudaMalloc(&h->sparse.flags[1], n);
    if (e == cudaSuccess) e = cudaMalloc(&h->sparse.list, n * sizeof(int32_t));
    if (e == cudaSuccess) e = cudaMalloc(&h->sparse.count, sizeof(int32_t));
    if (e != cudaSuccess) {
        h->sparse_on = false;
        return cuda_fail(e, "active-tile allocation");
    }
    h->sparse.background = background;
    h->sparse.tile_w = tile_w;
    h->sparse.tile_h = tilesize;
    h->sparse.tiles_x = tx;
    h->sparse.tiles_y = ty;
    h->sparse_on = true;
    h->sparse_dirty = true;
    return GBCA_OK;
}

int gbca_snapshot(gbca_handle* h, int64_t* ticket) {
    if (!h || !ticket) return fail(GBCA_ERR_ARGUMENT, "null handle or ticket");
    const size_t row = (size_t)h->d.n1 * h->esize, bytes = row * (size_t)h->d.n2;
    if (!h->copy_stream) GBCA_CUDA(cudaStreamCreateWithFlags(&h->copy_stream, cudaStreamNonBlocking), "copy stream");
    gbca_handle::Snapshot* sn = nullptr;
    for (auto& x : h->snaps)
        if (!x.busy) {
            sn = &x;
            break;
        }
    if (!sn) {
        if (h->snaps.size() >= (size_t)GBCA_MAX_SNAPSHOTS)
            return fail(GBCA_ERR_BUSY, "%d snapshots are waiting to be fetched", GBCA_MAX_SNAPSHOTS);
        h->snaps.emplace_back();
        sn = &h->snaps.back();
        cudaError_t e = cudaMalloc(&sn->dev, bytes);
        if (e == cudaSuccess) e = cudaMallocHost(&sn->host, bytes);
        if (e == cudaSuccess) e = cudaEventCreateWithFlags(&sn->staged, cudaEventDisableTiming);
        if (e == cudaSuccess) e = cudaEventCreateWithFlags(&sn->done, cudaEventDisableTiming);
        if (e != cudaSuccess) {
            cudaFree(sn->dev);
            if (sn->host) cudaFreeHost(sn->host);
            if (sn->staged) cudaEventDestroy(sn->staged);
            if (sn->done) cudaEventDestroy(sn->done);
            h->snaps.pop_back();
            cudaGetLastError();
            return e == cudaErrorMemoryAllocation ? fail(GBCA_ERR_OUT_OF_MEMORY, "snapshot buffers of %zu bytes", bytes)
                                                  : cuda_fail(e, "snapshot set-up");
        }
    }
    // stage on the device behind the queued steps, then copy out on the second stream, so
    // the sweep goes on while the copy runs
    GBCA_CUDA(cudaMemcpy2DAsync(sn->dev, row, h->buf[h->cur], (size_t)h->pitch, row, (size_t)h->d.n2,
                                cudaMemcpyDeviceToDevice, h->stream),
              "snapshot staging");
    GBCA_CUDA(cudaEventRecord(sn->staged, h->stream), "snapshot");
    GBCA_CUDA(cudaStreamWaitEvent(h->copy_stream, sn->staged, 0), "snapshot");
    GBCA_CUDA(cudaMemcpyAsync(sn->host, sn->dev, bytes, cudaMemcpyDeviceToHost, h->copy_stream), "snapshot copy");
    GBCA_CUDA(cudaEventRecord(sn->done, h->copy_stream), "snapshot");
    sn->busy = true;
    sn->ticket = h->next_ticket++;
    *ticket = sn->ticket;
    return GBCA_OK;
}

int gbca_snapshot_fetch(gbca_handle* h, int64_t ticket, void* host, size_t nbytes) {
    if (!h || !host) return fail(GBCA_ERR_ARGUMENT, "null handle or buffer");
    const size_t bytes = (size_t)h->d.n1 * h->esize * (size_t)h->d.n2;
    if (nbytes != bytes) return fail(GBCA_ERR_STATE, "the buffer has %zu bytes, the lattice needs %zu", nbytes, bytes);
    for (auto& sn : h->snaps) {
        if (!sn.busy || sn.ticket != ticket) continue;
        GBCA_CUDA(cudaEventSynchronize(sn.done), "snapshot fetch");
        std::memcpy(host, sn.host, bytes);
        sn.busy = false;
        return GBCA_OK;
    }
    return fail(GBCA_ERR_ARGUMENT, "no pending snapshot %lld", (long long)ticket);
}

int gbca_summaries(gbca_handle* h, int64_t* counts, int32_t nvals, int64_t* other, double* morans) {
    if (!h) return fail(GBCA_ERR_ARGUMENT, "null handle");
    if (h->d.rule == GBCA_RULE_LENIA) return fail(GBCA_ERR_UNSUPPORTED, "summaries need an Int8 state");
    if (nvals < 0 || nvals > 128) return fail(GBCA_ERR_ARGUMENT, "nvals must be in 0:128, got %d", nvals);
    GBCA_CUDA(gbca::launch_measures((const int8_t*)h->buf[h->cur], h->d.n1, h->d.n2, h->pitch, h->d.boundary[0],
                                    h->d.boundary[1], h->acc, h->nsm, h->stream),
              "summaries launch");
    GBCA_CUDA(cudaMemcpyAsync(h->acc_host, h->acc, gbca::kMeasureWords * sizeof(unsigned long long),
                              cudaMemcpyDeviceToHost, h->stream),
              "summaries copy");
    GBCA_CUDA(cudaStreamSynchronize(h->stream), "summaries");
    gbca::finish_measures(h->acc_host, h->d.n1 * h->d.n2, counts, nvals, other, morans);
    return GBCA_OK;
}

int gbca_set_stream(gbca_handle* h, void* stream) {
    if (!h) return fail(GBCA_ERR_ARGUMENT, "null handle");
    cudaStream_t next = stream ? (cudaStream_t)stream : h->own_stream;
    GBCA_CUDA(cudaStreamSynchronize(h->stream), "set_stream");
    h->stream = next;
    return GBCA_OK;
}

int64_t gbca_kernel_launches(void) { return gbca::launches_so_far(); }

int gbca_set_slab(gbca_handle* h, int64_t col0, int64_t n2_global) {
    if (!h) return fail(GBCA_ERR_ARGUMENT, "null handle");
    if (h->d.rule == GBCA_RULE_LENIA || h->d.rule == GBCA_RULE_SI_FIELD)
        return fail(GBCA_ERR_UNSUPPORTED, "slabs run rules without kernel fields (Life, Generations, forest fire)");
    if (h->sparse_on) return fail(GBCA_ERR_UNSUPPORTED, "a slab of a larger lattice runs dense sweeps only");
    if (n2_global < h->d.n2)
        return fail(GBCA_ERR_ARGUMENT, "the larger lattice (%lld columns) must hold the slab's %lld",
                    (long long)n2_global, (long long)h->d.n2);
    if (col0 <= -n2_global || col0 >= n2_global)
        return fail(GBCA_ERR_ARGUMENT, "the slab's first column %lld must lie in (-%lld, %lld)", (long long)col0,
                    (long long)n2_global, (long long)n2_global);
    if (h->d.n1 > INT64_MAX / n2_global) return fail(GBCA_ERR_ARGUMENT, "the larger lattice is too large");
    GBCA_CUDA(cudaStreamSynchronize(h->stream), "set_slab");
    h->slab_on = !(col0 == 0 && n2_global == h->d.n2);
    h->slab = gbca::SlabPlace{col0, n2_global};
    return GBCA_OK;
}

int gbca_slab_sums(gbca_handle* h, int64_t j_lo, int64_t j_hi, int64_t* sums) {
    if (!h || !sums) return fail(GBCA_ERR_ARGUMENT, "null handle or output");
    if (h->d.rule == GBCA_RULE_LENIA) return fail(GBCA_ERR_UNSUPPORTED, "summaries need an Int8 state");
    if (j_lo < 0 || j_hi > h->d.n2 || j_lo > j_hi)
        return fail(GBCA_ERR_ARGUMENT, "columns %lld:%lld lie outside 0:%lld", (long long)j_lo, (long long)j_hi,
                    (long long)h->d.n2);
    GBCA_CUDA(gbca::launch_measures((const int8_t*)h->buf[h->cur], h->d.n1, h->d.n2, h->pitch, h->d.boundary[0],
                                    h->d.boundary[1], h->acc, h->nsm, h->stream, j_lo, j_hi),
              "slab sums launch");
    GBCA_CUDA(cudaMemcpyAsync(h->acc_host, h->acc, gbca::kMeasureWords * sizeof(unsigned long long),
                              cudaMemcpyDeviceToHost, h->stream),
              "slab sums copy");
    GBCA_CUDA(cudaStreamSynchronize(h->stream), "slab sums");
    for (int k = 0; k < gbca::kMeasureWords; ++k) sums[k] = (int64_t)h->acc_host[k];
    return GBCA_OK;
}

int gbca_device_state(gbca_handle* h, void** dptr, int64_t* pitch) {
    if (!h || !dptr) return fail(GBCA_ERR_ARGUMENT, "null handle or output");
    h->sparse_dirty = true;  // the caller may write through the pointer
    *dptr = h->buf[h->cur];
    if (pitch) *pitch = h->pitch;
    return GBCA_OK;
}

}  // extern "C"
