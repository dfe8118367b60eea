// server.cu — a device-resident request loop with continuous batching.
//
// Clients submit simulation requests (an Int8 problem, its initial state, a step count and
// parameters) at any time; a scheduler thread owns the GPU and returns each request's
// summary statistics (state counts and Moran's I, src/measures.jl) as soon as it finishes.
//
//  * Admission by HBM budget: request states live in one device arena of a fixed size; a
//    request is admitted, in arrival order, when its two buffers fit, and its memory is
//    released the moment it finishes. A request larger than the whole arena is refused.
//  * Continuous batching, event driven: large requests run on `max_big` stream lanes in chunks
//    of about big_chunk_us (default kChunkSeconds) of estimated GPU time (temporally blocked multi-CTA sweeps; the
//    last chunk ends with the request's summaries); small requests run together, each up to
//    `chunk_steps` steps (fewer for larger lattices, so that no launch outlasts about
//    kSmallLaunchSeconds of one CTA's work) in persistent ensemble launches (ensemble.cu; one
//    CTA per request) on their own stream, back to back. Every launch ends with an event and a host
//    callback that wakes the scheduler, which then collects what finished, frees its memory,
//    admits waiting requests and refills the idle lane or the small stream at once: no lane
//    waits for another, and no iteration-wide barrier holds the device.
//  * Large requests are picked shortest estimated remaining time first, aged by their time in
//    the system (so none starves), and lanes are filled only while the chunks in flight
//    occupy at most kFillCap GPUs' worth of tiles: a long forest fire no longer holds a lane
//    from start to end while short requests queue behind it, and a dozen lattices that each
//    fill the GPU no longer share it sixteen ways.
//  * A request's initial state is uploaded or generated on the stream that then runs it, so
//    its first step is ordered after its state.
//  * Results are exact: a request's steps, draws and summaries are those it would get alone
//    (the draws depend only on its seed, cell and time).
// The scheduler never waits on the device inside a kernel: it polls events on the host, so
// there is no device-side spin to bound.
#include <algorithm>
#include <atomic>
#include <chrono>
#include <condition_variable>
#include <cstdarg>
#include <cstdio>
#include <cstring>
#include <deque>
#include <map>
#include <mutex>
#include <numeric>
#include <string>
#include <thread>
#include <vector>

#include "ensemble.cuh"
#include "gbca_internal.cuh"
#include "measures.cuh"

namespace gbca {

namespace {

size_t align256(size_t x) { return (x + 255) / 256 * 256; }

// First-fit allocator over a device arena (offsets only; the host owns the books).
class Arena {
  public:
    explicit Arena(size_t cap = 0) { reset(cap); }
    void reset(size_t cap) {
        free_.clear();
        cap_ = cap;
        if (cap) free_[0] = cap;
    }
    bool alloc(size_t n, size_t* off) {
        for (auto it = free_.begin(); it != free_.end(); ++it) {
            if (it->second >= n) {
                *off = it->first;
                const size_t rest = it->second - n, at = it->first + n;
                free_.erase(it);
                if (rest) free_[at] = rest;
                return true;
            }
        }
        return false;
    }
    void release(size_t off, size_t n) {
        auto it = free_.emplace(off, n).first;
        auto next = std::next(it);
        if (next != free_.end() && it->first + it->second == next->first) {
            it->second += next->second;
            free_.erase(next);
        }
        if (it != free_.begin()) {
            auto prev = std::prev(it);
            if (prev->first + prev->second == it->first) {
                prev->second += it->second;
                free_.erase(it);
            }
        }
    }
    size_t capacity() const { return cap_; }

  private:
    std::map<size_t, size_t> free_;
    size_t cap_ = 0;
};

struct Request {
    uint64_t id = 0;
    gbca_desc d;
    std::vector<int8_t> u0;  // empty: zeros or a soup
    double density = 0.0;
    uint64_t init_seed = 0;
    int64_t t0 = 0, nsteps = 0, done = 0;
    double params[2] = {0.0, 0.0};
    size_t off = 0, bytes = 0;
    int64_t pitch = 0;
    int cur = 0;
    bool big = false;
    bool fresh = true;  // the initial state is still to be written into the arena
    bool valid = true;  // every initial state is one the rule produces
    double t_submit = 0.0, t_admit = 0.0;
};

// Chunks of large requests: about this much estimated GPU time each unless the configuration
// says otherwise, and chunks in flight holding at most this many GPUs' worth of tiles.
constexpr double kChunkSeconds = 4e-3;
constexpr double kFillCap = 2.0;
// A persistent launch of small requests lasts as long as its slowest instance (one CTA each), and
// requests arriving meanwhile wait for it: each instance takes about this much of its CTA's time
// per launch (at most chunk_steps steps).
constexpr double kSmallLaunchSeconds = 1.5e-3;

int sfail(int code, const char* fmt, ...) {
    char msg[512];
    va_list ap;
    va_start(ap, fmt);
    vsnprintf(msg, sizeof msg, fmt, ap);
    va_end(ap);
    set_last_error(msg);
    return code;
}

}  // namespace

}  // namespace gbca

using namespace gbca;

struct gbca_server {
    gbca_server_config cfg;
    int device = 0;
    int8_t* arena_base = nullptr;
    Arena arena;
    std::mutex mu;
    std::condition_variable cv;
    std::deque<Request*> inbox;
    std::deque<gbca_result> outbox;
    std::thread th;
    bool stopping = false;
    bool dead = false;
    uint64_t next_id = 1;
    std::chrono::steady_clock::time_point t_start;
    int64_t queued = 0, active_n = 0;
    // scheduler-owned device resources
    cudaStream_t s_small = nullptr;
    std::vector<cudaStream_t> s_big;
    EnsInstance* d_inst = nullptr;
    int* d_order = nullptr;
    int* d_counter = nullptr;
    EnsSummary* d_out = nullptr;
    int* d_cur = nullptr;
    EnsSummary* h_out = nullptr;
    int* h_cur = nullptr;
    int cap_small = 0;
    unsigned long long* d_acc = nullptr;
    unsigned long long* h_acc = nullptr;
    int grid = 0;
    std::vector<cudaEvent_t> ev_big;  // end of each lane's request
    cudaEvent_t ev_small = nullptr;    // end of the small requests' launch in flight
    std::atomic<uint64_t> signals{0};  // completions reported by host callbacks
    // occupancy (under mu): seconds each lane and the small stream had work in flight, chunks run
    std::vector<double> lane_busy;
    double small_busy = 0.0;
    int64_t chunks = 0;

    double now() const {
        return std::chrono::duration<double>(std::chrono::steady_clock::now() - t_start).count();
    }
};

namespace {

gbca_result make_result(const Request* r, int status, double t_done) {
    gbca_result res;
    std::memset(&res, 0, sizeof res);
    res.id = r->id;
    res.status = status;
    res.morans = __builtin_nan("");
    res.t_submit = r->t_submit;
    res.t_admit = r->t_admit;
    res.t_done = t_done;
    return res;
}

bool grow_small(gbca_server* S, int need) {
    if (need <= S->cap_small) return true;
    int cap = std::max(need, 2 * S->cap_small + 64);
    cudaFree(S->d_inst);
    cudaFree(S->d_order);
    cudaFree(S->d_out);
    cudaFree(S->d_cur);
    if (S->h_out) cudaFreeHost(S->h_out);
    if (S->h_cur) cudaFreeHost(S->h_cur);
    S->d_inst = nullptr;
    S->d_order = S->d_cur = nullptr;
    S->d_out = S->h_out = nullptr;
    S->h_cur = nullptr;
    cudaError_t e = cudaMalloc(&S->d_inst, sizeof(EnsInstance) * cap);
    if (e == cudaSuccess) e = cudaMalloc(&S->d_order, sizeof(int) * cap);
    if (e == cudaSuccess) e = cudaMalloc(&S->d_out, sizeof(EnsSummary) * cap);
    if (e == cudaSuccess) e = cudaMalloc(&S->d_cur, sizeof(int) * cap);
    if (e == cudaSuccess) e = cudaMallocHost(&S->h_out, sizeof(EnsSummary) * cap);
    if (e == cudaSuccess) e = cudaMallocHost(&S->h_cur, sizeof(int) * cap);
    if (e != cudaSuccess) return false;
    S->cap_small = cap;
    return true;
}

EnsInstance small_instance(const Request* r, int64_t steps, bool last) {
    EnsInstance I;
    std::memset(&I, 0, sizeof I);
    const gbca_desc& d = r->d;
    I.n1 = d.n1;
    I.n2 = d.n2;
    I.pitch = r->pitch;
    I.off[0] = (int64_t)r->off;
    I.off[1] = (int64_t)(r->off + r->bytes / 2);
    I.t0 = r->t0 + r->done;
    I.nsteps = steps;
    I.birth = d.birth;
    I.survive = d.survive;
    I.seed = d.seed;
    if (d.rule == GBCA_RULE_FOREST_FIRE) {
        I.thr_p = gbca_threshold(r->params[0], d.params_f32);
        I.thr_f = gbca_threshold(r->params[1], d.params_f32);
    }
    I.rule = d.rule;
    I.nbhd = d.nbhd;
    I.radius = d.radius;
    I.states = d.states;
    I.params_f32 = d.params_f32;
    I.bnd0 = d.boundary[0];
    I.bnd1 = d.boundary[1];
    I.cval0 = d.boundary[0] == GBCA_CONSTANT ? (int32_t)d.constant[0] : 0;
    I.cval1 = d.boundary[1] == GBCA_CONSTANT ? (int32_t)d.constant[1] : 0;
    I.cur = r->cur;
    I.small = ensemble_fits_smem(d) ? 1 : 0;
    I.depth = ensemble_depth(d, 0);
    I.summarize = last ? 1 : 0;
    return I;
}

// Estimated sweep rate of a large request (cell-updates per second on one GB300): the forest
// fire is bound by its Philox draws, the bit-sliced Life and Generations kernels by their
// counting (by r), the general kernel by its per-cell loads.
double est_rate(const gbca_desc& d) {
    if (d.rule == GBCA_RULE_FOREST_FIRE) return d.nbhd == GBCA_VON_NEUMANN && d.radius == 1 ? 3.5e11 : 5e10;
    if (d.rule == GBCA_RULE_LIFE && d.nbhd == GBCA_MOORE && d.radius <= 7) return 4e12 / d.radius;
    if (d.rule == GBCA_RULE_GENERATIONS && d.nbhd == GBCA_MOORE && d.radius <= 2 && d.states <= 8)
        return 2e12 / d.radius;
    return 1e11 / (d.radius * d.radius);
}

// The share of the GPU one sweep of the request occupies (its tiles over the resident CTA
// slots), at most 1: a forest-fire tile is 256 x ~158 cells, two per SM; a bit-sliced tile up
// to 1024 x 216 cells.
double est_fill(const gbca_desc& d) {
    const double cells = (double)d.n1 * (double)d.n2;
    const double full = d.rule == GBCA_RULE_FOREST_FIRE ? 1.2e7 : 6e7;
    return cells >= full ? 1.0 : cells / full;
}

// Steps of a small request per persistent launch: kSmallLaunchSeconds of one CTA at its
// estimated rate (the forest fire's Philox draws, the other rules' byte-per-cell updates), at
// least 1 and at most chunk_steps.
int64_t small_chunk(const gbca_desc& d, int64_t chunk_steps) {
    const double cta_rate = d.rule == GBCA_RULE_FOREST_FIRE ? 3e8 : 6e8;
    const int64_t s = (int64_t)(kSmallLaunchSeconds * cta_rate / ((double)d.n1 * (double)d.n2));
    return s < 1 ? 1 : (s > chunk_steps ? chunk_steps : s);
}

double est_remaining_s(const Request* r) {
    return (double)r->d.n1 * (double)r->d.n2 * (double)(r->nsteps - r->done) / est_rate(r->d);
}

// Admit pending requests in arrival order while the arena has room; the state is initialised
// later, on the stream that runs the request.
void admit(gbca_server* S, std::deque<Request*>& pending, std::vector<Request*>& admitted,
           std::vector<gbca_result>& done) {
    while (!pending.empty()) {
        Request* r = pending.front();
        const gbca_desc& d = r->d;
        r->big = d.n1 * d.n2 > (int64_t)S->cfg.big_cells;
        r->pitch = r->big ? (d.n1 + 127) / 128 * 128 : d.n1;
        const size_t one = align256((size_t)(r->pitch * d.n2));
        r->bytes = 2 * one;
        if (r->bytes > S->arena.capacity()) {
            done.push_back(make_result(r, GBCA_ERR_OUT_OF_MEMORY, S->now()));
            pending.pop_front();
            delete r;
            continue;
        }
        if (!S->arena.alloc(r->bytes, &r->off)) break;
        r->cur = 0;
        r->done = 0;
        r->fresh = true;
        r->t_admit = S->now();
        admitted.push_back(r);
        pending.pop_front();
    }
}

// Writes a request's initial state into its first buffer on stream st.
cudaError_t init_state(gbca_server* S, Request* r, cudaStream_t st) {
    r->fresh = false;
    const gbca_desc& d = r->d;
    int8_t* buf = S->arena_base + r->off;
    if (!r->u0.empty()) {
        // a pageable source is staged before the call returns, so it can go at once
        const cudaError_t e = cudaMemcpy2DAsync(buf, (size_t)r->pitch, r->u0.data(), (size_t)d.n1, (size_t)d.n1,
                                                (size_t)d.n2, cudaMemcpyHostToDevice, st);
        std::vector<int8_t>().swap(r->u0);
        return e;
    }
    if (r->density > 0.0) {
        return launch_soup(buf, d.n1, d.n2, r->pitch, r->density, r->init_seed, S->grid, st);
    }
    return cudaMemsetAsync(buf, 0, r->bytes / 2, st);
}

void CUDART_CB on_done(void* p) {
    gbca_server* S = (gbca_server*)p;
    S->signals.fetch_add(1, std::memory_order_release);
    S->cv.notify_all();
}

void scheduler(gbca_server* S) {
    cudaSetDevice(S->device);
    std::deque<Request*> pending;
    std::vector<Request*> waiting_big;  // admitted large requests between chunks (or not started)
    std::vector<Request*> smalls;       // admitted small requests
    std::vector<Request*> batch;        // the small requests of the launch in flight
    std::vector<int64_t> batch_steps;
    const int nlanes = (int)S->s_big.size();
    std::vector<Request*> lane((size_t)nlanes, nullptr);
    std::vector<int64_t> lane_steps((size_t)nlanes, 0);
    std::vector<double> lane_start((size_t)nlanes, 0.0), lane_fill((size_t)nlanes, 0.0);
    std::vector<double> busy_add((size_t)nlanes, 0.0);
    double small_start = 0.0, small_add = 0.0;
    int64_t chunks_add = 0;
    bool small_busy = false;
    std::vector<gbca_result> done;
    uint64_t seen = 0;
    for (;;) {
        const bool busy = small_busy || std::any_of(lane.begin(), lane.end(), [](Request* r) { return r; });
        {
            std::unique_lock<std::mutex> lock(S->mu);
            while (S->inbox.empty() && pending.empty() && waiting_big.empty() && smalls.empty() && !busy &&
                   !S->stopping)
                S->cv.wait_for(lock, std::chrono::milliseconds(50));
            while (!S->inbox.empty()) {
                pending.push_back(S->inbox.front());
                S->inbox.pop_front();
            }
            if (S->stopping && pending.empty() && waiting_big.empty() && smalls.empty() && !busy) break;
        }
        cudaError_t e = cudaSuccess;
        bool progress = false;
        const double t = S->now();
        std::vector<Request*> finished;
        // 1. lanes whose chunk is done: the request goes back to the queue, or its summaries out
        for (int j = 0; j < nlanes && e == cudaSuccess; ++j) {
            Request* r = lane[(size_t)j];
            if (!r) continue;
            const cudaError_t q = cudaEventQuery(S->ev_big[(size_t)j]);
            if (q == cudaErrorNotReady) continue;
            if (q != cudaSuccess) {
                e = q;
                break;
            }
            lane[(size_t)j] = nullptr;
            busy_add[(size_t)j] += t - lane_start[(size_t)j];
            progress = true;
            r->done += lane_steps[(size_t)j];
            r->valid = true;  // the rule's own states from here on
            if (r->done < r->nsteps) {
                waiting_big.push_back(r);
                continue;
            }
            // a tile copy that gave up its wait left a tile unwritten: the result is not valid
            gbca_result res = make_result(r, fire_tma_timeouts_take() ? GBCA_ERR_TIMEOUT : GBCA_OK, t);
            finish_measures(S->h_acc + (size_t)j * kMeasureWords, r->d.n1 * r->d.n2, res.counts, kEnsCounts,
                            &res.other, &res.morans);
            done.push_back(res);
            finished.push_back(r);
        }
        // 2. the small requests' launch
        if (e == cudaSuccess && small_busy) {
            const cudaError_t q = cudaEventQuery(S->ev_small);
            if (q == cudaSuccess) {
                small_busy = false;
                small_add += t - small_start;
                progress = true;
                for (size_t j = 0; j < batch.size(); ++j) {
                    Request* r = batch[j];
                    r->cur = S->h_cur[j];
                    r->done += batch_steps[j];
                    if (r->done < r->nsteps) continue;
                    gbca_result res = make_result(r, GBCA_OK, t);
                    const long long* w = S->h_out[j].w;
                    const int64_t ncell = r->d.n1 * r->d.n2;
                    int64_t inrange = 0;
                    for (int v = 0; v < kEnsCounts; ++v) {
                        res.counts[v] = w[v];
                        inrange += w[v];
                    }
                    res.other = ncell - inrange;
                    res.morans = morans_from_sums(w[kEnsCounts + 1], w[kEnsCounts + 2], w[kEnsCounts + 3],
                                                  w[kEnsCounts + 4], w[kEnsCounts + 5], ncell);
                    done.push_back(res);
                    finished.push_back(r);
                    smalls.erase(std::find(smalls.begin(), smalls.end(), r));
                }
                batch.clear();
            } else if (q != cudaErrorNotReady) {
                e = q;
            }
        }
        for (Request* r : finished) {
            S->arena.release(r->off, r->bytes);
            delete r;
        }
        // 3. admission into the memory just freed
        if (e == cudaSuccess) {
            std::vector<Request*> admitted;
            admit(S, pending, admitted, done);
            for (Request* r : admitted) (r->big ? waiting_big : smalls).push_back(r);
            progress = progress || !admitted.empty();
        }
        // 4. idle lanes take the next chunk of the large request with the shortest estimated
        //    remaining time (aged by its time in the system), while the chunks in flight fill at
        //    most kFillCap GPUs
        for (int j = 0; j < nlanes && e == cudaSuccess && !waiting_big.empty(); ++j) {
            if (lane[(size_t)j]) continue;
            double fill = 0.0;
            for (int k = 0; k < nlanes; ++k)
                if (lane[(size_t)k]) fill += lane_fill[(size_t)k];
            const double now = S->now();
            auto key = [&](const Request* r) { return est_remaining_s(r) - (now - r->t_admit); };
            auto best = std::min_element(waiting_big.begin(), waiting_big.end(),
                                         [&](const Request* a, const Request* b) { return key(a) < key(b); });
            Request* r = *best;
            if (fill > 0.0 && fill + est_fill(r->d) > kFillCap) break;
            waiting_big.erase(best);
            const double cells = (double)r->d.n1 * (double)r->d.n2;
            const int64_t rem = r->nsteps - r->done;
            const double chunk_s = S->cfg.big_chunk_us > 0 ? S->cfg.big_chunk_us * 1e-6 : kChunkSeconds;
            int64_t steps = (int64_t)(est_rate(r->d) * chunk_s / cells);
            if (steps < S->cfg.chunk_steps) steps = S->cfg.chunk_steps;
            if (steps > rem) steps = rem;
            cudaStream_t st = S->s_big[(size_t)j];
            if (r->fresh) e = init_state(S, r, st);
            int8_t* const bufs[2] = {S->arena_base + r->off, S->arena_base + r->off + r->bytes / 2};
            if (e == cudaSuccess)
                e = sweep_int8(r->d, r->pitch, bufs, &r->cur, r->t0 + r->done, steps, r->params, st, r->valid);
            if (steps == rem) {  // the last chunk: the request's summaries
                unsigned long long* acc = S->d_acc + (size_t)j * kMeasureWords;
                if (e == cudaSuccess)
                    e = launch_measures(bufs[r->cur], r->d.n1, r->d.n2, r->pitch, r->d.boundary[0], r->d.boundary[1],
                                        acc, S->grid / 4 > 0 ? S->grid / 4 : 1, st);
                if (e == cudaSuccess)
                    e = cudaMemcpyAsync(S->h_acc + (size_t)j * kMeasureWords, acc,
                                        kMeasureWords * sizeof(unsigned long long), cudaMemcpyDeviceToHost, st);
            }
            if (e == cudaSuccess) e = cudaEventRecord(S->ev_big[(size_t)j], st);
            if (e == cudaSuccess) e = cudaLaunchHostFunc(st, on_done, S);
            lane[(size_t)j] = r;
            lane_steps[(size_t)j] = steps;
            lane_start[(size_t)j] = now;
            lane_fill[(size_t)j] = est_fill(r->d);
            ++chunks_add;
            progress = true;
        }
        // 5. the small requests, chunk_steps at a time, in one persistent launch
        if (e == cudaSuccess && !small_busy && !smalls.empty()) {
            if (!grow_small(S, (int)smalls.size())) e = cudaErrorMemoryAllocation;
            batch = smalls;
            batch_steps.assign(batch.size(), 0);
            std::vector<EnsInstance> inst(batch.size());
            std::vector<int64_t> work(batch.size());
            for (size_t j = 0; j < batch.size() && e == cudaSuccess; ++j) {
                Request* r = batch[j];
                if (r->fresh) e = init_state(S, r, S->s_small);
                const int64_t rem = r->nsteps - r->done, cap = small_chunk(r->d, S->cfg.chunk_steps);
                batch_steps[j] = rem < cap ? rem : cap;
                inst[j] = small_instance(r, batch_steps[j], batch_steps[j] == rem);
                work[j] = r->d.n1 * r->d.n2 * batch_steps[j];
            }
            std::vector<int> order(batch.size());
            std::iota(order.begin(), order.end(), 0);
            std::stable_sort(order.begin(), order.end(), [&](int a, int b) { return work[a] > work[b]; });
            if (e == cudaSuccess)
                e = cudaMemcpyAsync(S->d_inst, inst.data(), sizeof(EnsInstance) * inst.size(), cudaMemcpyHostToDevice,
                                    S->s_small);
            if (e == cudaSuccess)
                e = cudaMemcpyAsync(S->d_order, order.data(), sizeof(int) * order.size(), cudaMemcpyHostToDevice,
                                    S->s_small);
            if (e == cudaSuccess)
                e = launch_ensemble(S->d_inst, S->d_order, (int)inst.size(), S->d_counter, S->arena_base, S->d_out,
                                    S->d_cur, S->grid, S->s_small);
            if (e == cudaSuccess)
                e = cudaMemcpyAsync(S->h_out, S->d_out, sizeof(EnsSummary) * inst.size(), cudaMemcpyDeviceToHost,
                                    S->s_small);
            if (e == cudaSuccess)
                e = cudaMemcpyAsync(S->h_cur, S->d_cur, sizeof(int) * inst.size(), cudaMemcpyDeviceToHost, S->s_small);
            if (e == cudaSuccess) e = cudaEventRecord(S->ev_small, S->s_small);
            if (e == cudaSuccess) e = cudaLaunchHostFunc(S->s_small, on_done, S);
            small_busy = e == cudaSuccess;
            small_start = S->now();
            progress = true;
        }
        if (e != cudaSuccess) {
            // the device failed: every admitted and queued request fails with it
            cudaGetLastError();
            std::vector<Request*> all(pending.begin(), pending.end());
            all.insert(all.end(), waiting_big.begin(), waiting_big.end());
            all.insert(all.end(), smalls.begin(), smalls.end());
            for (Request* r : lane)
                if (r) all.push_back(r);
            for (Request* r : all) {
                done.push_back(make_result(r, GBCA_ERR_CUDA, S->now()));
                delete r;
            }
            pending.clear();
            waiting_big.clear();
            smalls.clear();
            batch.clear();
            std::fill(lane.begin(), lane.end(), nullptr);
            small_busy = false;
            std::lock_guard<std::mutex> lock(S->mu);
            S->dead = true;
            for (auto& res : done) S->outbox.push_back(res);
            done.clear();
            S->stopping = true;
            continue;
        }
        {
            std::unique_lock<std::mutex> lock(S->mu);
            for (auto& res : done) S->outbox.push_back(res);
            done.clear();
            for (int j = 0; j < nlanes; ++j) {
                S->lane_busy[(size_t)j] += busy_add[(size_t)j];
                busy_add[(size_t)j] = 0.0;
            }
            S->small_busy += small_add;
            small_add = 0.0;
            S->chunks += chunks_add;
            chunks_add = 0;
            S->queued = (int64_t)(pending.size() + S->inbox.size());
            S->active_n = (int64_t)(waiting_big.size() + smalls.size() +
                                    std::count_if(lane.begin(), lane.end(), [](Request* r) { return r; }));
            if (!progress) {  // nothing finished or started: sleep until a launch ends or a request arrives
                const uint64_t now_signals = S->signals.load(std::memory_order_acquire);
                if (now_signals == seen && S->inbox.empty() && !S->stopping)
                    S->cv.wait_for(lock, std::chrono::milliseconds(1));
                seen = S->signals.load(std::memory_order_acquire);
            }
        }
    }
}

}  // namespace

extern "C" {

int gbca_server_start(const gbca_server_config* cfg, gbca_server** out) {
    if (!cfg || !out) return sfail(GBCA_ERR_ARGUMENT, "null configuration or output");
    *out = nullptr;
    if (cfg->hbm_budget < 4096 || cfg->chunk_steps < 1 || cfg->max_big < 1 || cfg->max_big > 64 ||
        cfg->big_cells < 0 || cfg->big_chunk_us < 0)
        return sfail(GBCA_ERR_ARGUMENT, "server configuration out of range");
    if (gbca_device_count() < 1) return sfail(GBCA_ERR_CUDA, "no CUDA device is visible");
    gbca_server* S = new gbca_server();
    S->cfg = *cfg;
    S->t_start = std::chrono::steady_clock::now();
    cudaGetDevice(&S->device);
    cudaError_t e = cudaMalloc(&S->arena_base, (size_t)cfg->hbm_budget);
    if (e == cudaSuccess) e = cudaStreamCreateWithFlags(&S->s_small, cudaStreamNonBlocking);
    S->s_big.assign((size_t)cfg->max_big, nullptr);
    for (auto& st : S->s_big)
        if (e == cudaSuccess) e = cudaStreamCreateWithFlags(&st, cudaStreamNonBlocking);
    S->ev_big.assign((size_t)cfg->max_big, nullptr);
    for (auto& ev : S->ev_big)
        if (e == cudaSuccess) e = cudaEventCreateWithFlags(&ev, cudaEventDisableTiming);
    if (e == cudaSuccess) e = cudaEventCreateWithFlags(&S->ev_small, cudaEventDisableTiming);
    if (e == cudaSuccess) e = cudaMalloc(&S->d_counter, sizeof(int));
    if (e == cudaSuccess) e = cudaMalloc(&S->d_acc, sizeof(unsigned long long) * kMeasureWords * cfg->max_big);
    if (e == cudaSuccess) e = cudaMallocHost(&S->h_acc, sizeof(unsigned long long) * kMeasureWords * cfg->max_big);
    if (e != cudaSuccess) {
        const bool oom = e == cudaErrorMemoryAllocation;
        cudaGetLastError();
        cudaFree(S->arena_base);
        cudaFree(S->d_counter);
        cudaFree(S->d_acc);
        if (S->h_acc) cudaFreeHost(S->h_acc);
        if (S->s_small) cudaStreamDestroy(S->s_small);
        for (auto st : S->s_big)
            if (st) cudaStreamDestroy(st);
        for (auto ev : S->ev_big)
            if (ev) cudaEventDestroy(ev);
        if (S->ev_small) cudaEventDestroy(S->ev_small);
        delete S;
        return oom ? sfail(GBCA_ERR_OUT_OF_MEMORY, "the server's HBM budget of %llu bytes cannot be allocated",
                           (unsigned long long)cfg->hbm_budget)
                   : sfail(GBCA_ERR_CUDA, "server start: %s", cudaGetErrorString(e));
    }
    S->arena.reset((size_t)cfg->hbm_budget);
    S->lane_busy.assign((size_t)cfg->max_big, 0.0);
    S->grid = ensemble_grid();
    S->th = std::thread(scheduler, S);
    *out = S;
    return GBCA_OK;
}

int gbca_server_submit(gbca_server* S, const gbca_desc* d, const void* u0, size_t nbytes, double init_density,
                       uint64_t init_seed, int64_t t0, int64_t nsteps, const double* params, int32_t nparams,
                       uint64_t* id) {
    if (!S || !d) return sfail(GBCA_ERR_ARGUMENT, "null server or problem");
    const int rc = gbca_check(d);
    if (rc != GBCA_OK) return rc;
    if (d->rule == GBCA_RULE_LENIA || d->rule == GBCA_RULE_SI_FIELD || d->scheme != GBCA_SYNCHRONOUS || d->radius > 8)
        return sfail(GBCA_ERR_UNSUPPORTED, "the server runs Int8 rules, Synchronous(), radius <= 8");
    if (nsteps < 0) return sfail(GBCA_ERR_ARGUMENT, "negative step count");
    if (d->rule == GBCA_RULE_FOREST_FIRE && (!params || nparams < 2))
        return sfail(GBCA_ERR_ARGUMENT, "the forest-fire rule needs parameters (p, f)");
    if (u0 && nbytes != (size_t)(d->n1 * d->n2))
        return sfail(GBCA_ERR_STATE, "the state has %zu bytes, the lattice %lld cells", nbytes,
                     (long long)(d->n1 * d->n2));
    if (!(init_density >= 0.0 && init_density <= 1.0))
        return sfail(GBCA_ERR_ARGUMENT, "initial density must be in [0, 1]");
    Request* r = new Request();
    r->d = *d;
    if (u0) {
        r->u0.assign((const int8_t*)u0, (const int8_t*)u0 + nbytes);
        const int nv = d->rule == GBCA_RULE_GENERATIONS ? d->states : (d->rule == GBCA_RULE_FOREST_FIRE ? 3 : 256);
        for (int8_t v : r->u0)
            if (v < 0 || v >= nv) {
                r->valid = false;
                break;
            }
    }
    r->density = init_density;
    r->init_seed = init_seed;
    r->t0 = t0;
    r->nsteps = nsteps;
    if (params && nparams >= 2) {
        r->params[0] = params[0];
        r->params[1] = params[1];
    }
    {
        std::lock_guard<std::mutex> lock(S->mu);
        if (S->stopping) {
            delete r;
            return sfail(GBCA_ERR_BUSY, "the server is stopping");
        }
        r->id = S->next_id++;
        r->t_submit = S->now();
        S->inbox.push_back(r);
        ++S->queued;
    }
    S->cv.notify_one();
    if (id) *id = r->id;
    return GBCA_OK;
}

int gbca_server_poll(gbca_server* S, gbca_result* out, int32_t max, int32_t* n) {
    if (!S || !n || (max > 0 && !out)) return sfail(GBCA_ERR_ARGUMENT, "null server or output");
    std::lock_guard<std::mutex> lock(S->mu);
    int32_t k = 0;
    while (k < max && !S->outbox.empty()) {
        out[k++] = S->outbox.front();
        S->outbox.pop_front();
    }
    *n = k;
    return GBCA_OK;
}

int gbca_server_status(gbca_server* S, int64_t* queued, int64_t* active, double* clock) {
    if (!S) return sfail(GBCA_ERR_ARGUMENT, "null server");
    std::lock_guard<std::mutex> lock(S->mu);
    if (queued) *queued = S->queued;
    if (active) *active = S->active_n;
    if (clock) *clock = S->now();
    return S->dead ? sfail(GBCA_ERR_CUDA, "the server stopped after a device failure") : GBCA_OK;
}

int gbca_server_stats(gbca_server* S, double* lane_busy_s, int32_t max_lanes, int32_t* nlanes, double* small_busy_s,
                      double* wall_s, int64_t* chunks) {
    if (!S || (max_lanes > 0 && !lane_busy_s)) return sfail(GBCA_ERR_ARGUMENT, "null server or output");
    std::lock_guard<std::mutex> lock(S->mu);
    const int32_t n = (int32_t)S->lane_busy.size();
    for (int32_t j = 0; j < n && j < max_lanes; ++j) lane_busy_s[j] = S->lane_busy[(size_t)j];
    if (nlanes) *nlanes = n;
    if (small_busy_s) *small_busy_s = S->small_busy;
    if (wall_s) *wall_s = S->now();
    if (chunks) *chunks = S->chunks;
    return GBCA_OK;
}

int gbca_server_stop(gbca_server* S) {
    if (!S) return GBCA_OK;
    {
        std::lock_guard<std::mutex> lock(S->mu);
        S->stopping = true;
    }
    S->cv.notify_all();
    if (S->th.joinable()) S->th.join();
    for (Request* r : S->inbox) delete r;
    cudaFree(S->arena_base);
    cudaFree(S->d_inst);
    cudaFree(S->d_order);
    cudaFree(S->d_counter);
    cudaFree(S->d_out);
    cudaFree(S->d_cur);
    cudaFree(S->d_acc);
    if (S->h_out) cudaFreeHost(S->h_out);
    if (S->h_cur) cudaFreeHost(S->h_cur);
    if (S->h_acc) cudaFreeHost(S->h_acc);
    if (S->s_small) cudaStreamDestroy(S->s_small);
    for (auto st : S->s_big)
        if (st) cudaStreamDestroy(st);
    for (auto ev : S->ev_big)
        if (ev) cudaEventDestroy(ev);
    if (S->ev_small) cudaEventDestroy(S->ev_small);
    delete S;
    return GBCA_OK;
}

}  // extern "C"
