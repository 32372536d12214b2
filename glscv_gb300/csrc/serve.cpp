// serve.cpp -- phaseCorrelate serving loop with resident reference spectra
// and continuous batching.
//
// A server owns one device arena (its whole HBM budget, reserved once), a set
// of slots (a CUDA stream, an event and a mapped pinned result buffer each),
// and native threads of two kinds:
//   * dispatchers (kDispatchers threads) admit queued requests in arrival
//     order as soon as a slot is free and the request's workspace fits in the
//     arena (looking a few requests past a head that does not fit yet), and
//     launch the request's whole pipeline on the slot's stream: host->device
//     copy of the frame, windowed row FFT, phase-only column kernel against
//     the resident reference spectrum (so 2 FFTs per request instead of 3),
//     inverse row FFT with the argmax, whose last block writes the FP64
//     centroid straight into the slot's result buffer;
//   * the completion poller watches the slots' events (queried without the
//     lock), stamps completion times, returns workspaces to the arena and
//     wakes the dispatchers.
// Several dispatchers issue the CUDA calls of different requests at once, so
// the host's call rate does not cap the request rate.
// Requests that arrive while others run are admitted as resources free up,
// so their kernels overlap on the device.  The kernels are deterministic, so
// a request's result does not depend on what runs beside it.
#include <algorithm>
#include <atomic>
#include <chrono>
#include <condition_variable>
#include <cstring>
#include <deque>
#include <mutex>
#include <new>
#include <thread>
#include <unordered_map>
#include <vector>

#include "arena.h"
#include "capi_internal.h"
#include "glsfft_internal.h"

using namespace glsfft;
using Clock = std::chrono::steady_clock;

namespace {

struct Reference {
    int rows = 0, cols = 0;
    size_t spec_off = 0, win_off = 0;
    bool has_window = false;
};

enum { REQ_QUEUED = 0, REQ_RUNNING = 1, REQ_DONE = 2, REQ_FAILED = 3 };

struct Request {
    int ref = 0;
    const float *frame = nullptr;  // host pointer, valid until completion
    bool direct = false;           // the row kernel reads `frame` itself
    int box = 5;
    // arrival: the scheduled arrival (latency counts from it); submitted: when
    // the request was queued; admitted: when a dispatcher took a slot and
    // workspace for it; launched: when its pipeline and event were issued;
    // done_at: when the poller saw the event complete
    Clock::time_point arrival, submitted, admitted, launched, done_at;
    int state = REQ_QUEUED;
    int status = GLSFFT_SUCCESS;
    int slot = -1;
    size_t ws_off = Arena::kFail;
    double result[5] = {0, 0, 0, 0, 0};
    double gpu_s = 0.0;   // device time from the start event to the done event
    double copy_s = 0.0;  // of which the frame's host-to-device copy
};

struct Slot {
    cudaStream_t stream = nullptr;
    cudaEvent_t start = nullptr;   // recorded before the frame's copy (timing)
    cudaEvent_t copied = nullptr;  // recorded after the frame's copy (timing)
    cudaEvent_t done = nullptr;   // recorded after the last launch (timing)
    double *h_result = nullptr;      // pinned and mapped, 8 doubles
    double *h_result_dev = nullptr;  // its device-side address
    long long ticket = -1;
    bool launched = false;  // the event of this ticket's pipeline is recorded
};

constexpr int kDispatchers = 3;

size_t workspace_bytes(int rows, int cols) {
    const size_t n = (size_t)rows * cols;
    // frame (float) | row-pass / column output (complex) | surface (float) | key | result
    return Arena::round_up(4 * n) + Arena::round_up(8 * n) + Arena::round_up(4 * n) + 256;
}

}  // namespace

struct glsfft_server_s {
    glsfft_context ctx = nullptr;
    int device = 0;
    char *d_base = nullptr;
    Arena arena;
    std::vector<Reference> refs;
    std::vector<Slot> slots;
    std::mutex mu;
    std::condition_variable cv_dispatch, cv_poll, cv_done;
    std::deque<long long> queue;
    std::unordered_map<long long, Request> reqs;
    long long next_ticket = 1;
    int in_flight = 0;
    bool direct_read = true;  // glsfft_server_set_frame_read
    bool stop = false;
    std::vector<std::thread> dispatchers;
    std::thread poller;
    // counters
    long long admitted = 0, completed = 0, failed = 0;
    long long peak_in_flight = 0, peak_queue = 0;
    size_t peak_arena = 0;
};

namespace {

// Launch one request's pipeline on its slot.  Called without the lock held.
int launch_request(glsfft_server srv, const Reference &ref, const Request &rq, Slot &slot) {
    const int rows = ref.rows, cols = ref.cols;
    const size_t n = (size_t)rows * cols;
    char *ws = srv->d_base + rq.ws_off;
    float *frame = reinterpret_cast<float *>(ws);
    float2 *f2 = reinterpret_cast<float2 *>(ws + Arena::round_up(4 * n));
    float *surface = reinterpret_cast<float *>(ws + Arena::round_up(4 * n) + Arena::round_up(8 * n));
    char *tail = ws + Arena::round_up(4 * n) + Arena::round_up(8 * n) + Arena::round_up(4 * n);
    auto *key = reinterpret_cast<unsigned long long *>(tail);  // argmax key, block counter
    const float2 *spec = reinterpret_cast<const float2 *>(srv->d_base + ref.spec_off);
    const float *win = ref.has_window ? reinterpret_cast<const float *>(srv->d_base + ref.win_off) : nullptr;
    cudaStream_t s = slot.stream;

    // five calls: the frame's upload, three launches (the POC column pass
    // zeroes the argmax key; the last block of the inverse row pass computes
    // the centroid and writes it into the slot's mapped pinned buffer), the event
    cudaError_t e = cudaEventRecord(slot.start, s);
    if (e == cudaSuccess && !rq.direct)
        e = cudaMemcpyAsync(frame, rq.frame, 4 * n, cudaMemcpyHostToDevice, s);
    if (e == cudaSuccess) e = cudaEventRecord(slot.copied, s);
    if (e != cudaSuccess) return cuda_status(e);
    PassArgs a{};
    // direct: the windowed row pass loads the page-locked host frame over the
    // host link itself (its device address is the host address under unified
    // addressing), so no copy-engine transfer precedes it
    a.in0 = rq.direct ? rq.frame : frame;
    a.out0 = f2;
    a.window = win;
    a.rows = rows;
    a.cols = cols;
    a.scale = 1.0f;
    a.tw = srv->ctx->d_tw;
    e = launch_rows(cols, win ? LD_R1W : LD_R1, ST_C2, a, 1, s);
    if (e != cudaSuccess) return cuda_status(e);
    PassArgs b{};
    b.in0 = spec;  // resident reference spectrum (already column-transformed)
    b.in1 = f2;
    b.out0 = f2;   // in place over the frame's row-pass output
    b.rows = rows;
    b.cols = cols;
    b.scale = 1.0f;
    b.flags = PF_F1_SPECTRUM;
    b.key = key;
    b.tw = srv->ctx->d_tw;
    b.pdl = 1;  // resident while the row pass drains
    e = launch_poc_cols(rows, b, s);
    if (e != cudaSuccess) return cuda_status(e);
    PassArgs c{};
    c.in0 = f2;
    c.out0 = surface;
    c.rows = rows;
    c.cols = cols;
    c.scale = 1.0f;
    c.flags = PF_SHIFT_ROWS | PF_SHIFT_COLS;
    c.key = key;
    c.tw = srv->ctx->d_tw;
    c.result = slot.h_result_dev;
    c.box = rq.box;
    c.pdl = 1;
    e = launch_rows(cols, LD_C2, ST_RE_ARGMAX, c, 1, s);
    if (e == cudaSuccess) e = cudaEventRecord(slot.done, s);
    return cuda_status(e);
}

void dispatcher_main(glsfft_server srv) {
    cudaSetDevice(srv->device);
    std::unique_lock<std::mutex> lock(srv->mu);
    constexpr size_t kLookahead = 8;
    while (!srv->stop) {
        bool progress = false;
        for (size_t qi = 0; qi < srv->queue.size() && qi < kLookahead;) {
            const long long ticket = srv->queue[qi];
            Request &rq = srv->reqs[ticket];
            const Reference ref = srv->refs[rq.ref];
            const size_t need = workspace_bytes(ref.rows, ref.cols);
            int free_slot = -1;
            for (int i = 0; i < (int)srv->slots.size(); i++)
                if (srv->slots[i].ticket < 0) {
                    free_slot = i;
                    break;
                }
            if (free_slot < 0) break;  // every slot busy: nothing more to admit now
            const size_t off = srv->arena.alloc(need);
            if (off == Arena::kFail) {
                qi++;  // look past a request that does not fit yet
                continue;
            }
            srv->queue.erase(srv->queue.begin() + qi);
            rq.ws_off = off;
            rq.slot = free_slot;
            rq.state = REQ_RUNNING;
            rq.admitted = Clock::now();
            Slot &slot = srv->slots[free_slot];
            slot.ticket = ticket;
            slot.launched = false;  // not pollable until its event is recorded
            srv->in_flight++;
            srv->admitted++;
            srv->peak_in_flight = std::max<long long>(srv->peak_in_flight, srv->in_flight);
            srv->peak_arena = std::max(srv->peak_arena, srv->arena.in_use());
            const Request snapshot = rq;
            lock.unlock();
            const int st = launch_request(srv, ref, snapshot, slot);
            lock.lock();
            if (st != GLSFFT_SUCCESS) {
                Request &r2 = srv->reqs[ticket];
                r2.state = REQ_FAILED;
                r2.status = st;
                r2.done_at = Clock::now();
                srv->arena.release(r2.ws_off);
                srv->slots[free_slot].ticket = -1;
                srv->in_flight--;
                srv->failed++;
                srv->cv_done.notify_all();
            } else {
                srv->reqs[ticket].launched = Clock::now();
                srv->slots[free_slot].launched = true;
            }
            srv->cv_poll.notify_one();
            progress = true;
        }
        if (!progress) srv->cv_dispatch.wait(lock);
    }
}

void poller_main(glsfft_server srv) {
    cudaSetDevice(srv->device);
    struct Watch {
        int slot;
        long long ticket;
        cudaEvent_t ev;
    };
    std::vector<Watch> watch;
    std::vector<cudaError_t> state;
    std::unique_lock<std::mutex> lock(srv->mu);
    for (;;) {
        if (srv->in_flight == 0) {
            if (srv->stop) break;
            srv->cv_poll.wait(lock);
            continue;
        }
        // the launched slots, then their events queried without the lock
        watch.clear();
        for (int i = 0; i < (int)srv->slots.size(); i++) {
            const Slot &slot = srv->slots[i];
            if (slot.ticket >= 0 && slot.launched) watch.push_back({i, slot.ticket, slot.done});
        }
        lock.unlock();
        state.resize(watch.size());
        bool any_done = false;
        for (size_t w = 0; w < watch.size(); w++) {
            state[w] = cudaEventQuery(watch[w].ev);
            any_done |= state[w] != cudaErrorNotReady;
        }
        if (!any_done) std::this_thread::yield();
        lock.lock();
        bool any = false;
        for (size_t w = 0; w < watch.size(); w++) {
            if (state[w] == cudaErrorNotReady) continue;
            Slot &slot = srv->slots[watch[w].slot];
            if (slot.ticket != watch[w].ticket) continue;
            Request &rq = srv->reqs[slot.ticket];
            rq.done_at = Clock::now();
            if (state[w] == cudaSuccess) {
                std::memcpy(rq.result, slot.h_result, sizeof(rq.result));
                float ms = 0.f;
                if (cudaEventElapsedTime(&ms, slot.start, slot.done) == cudaSuccess) rq.gpu_s = 1e-3 * ms;
                if (cudaEventElapsedTime(&ms, slot.start, slot.copied) == cudaSuccess) rq.copy_s = 1e-3 * ms;
                rq.state = REQ_DONE;
                srv->completed++;
            } else {
                cudaGetLastError();
                rq.state = REQ_FAILED;
                rq.status = GLSFFT_ERROR_CUDA;
                srv->failed++;
            }
            srv->arena.release(rq.ws_off);
            slot.ticket = -1;
            srv->in_flight--;
            any = true;
        }
        if (any) {
            srv->cv_dispatch.notify_all();
            srv->cv_done.notify_all();
        }
    }
}

// Whether a kernel on the server's device may read `frame` directly: page-
// locked host memory whose device address is its host address.
bool frame_readable(glsfft_server srv, const float *frame) {
    cudaPointerAttributes at{};
    if (cudaPointerGetAttributes(&at, frame) != cudaSuccess) {
        cudaGetLastError();
        return false;
    }
    (void)srv;
    return at.type == cudaMemoryTypeHost && at.devicePointer == frame;
}

long long submit_locked(glsfft_server srv, int ref_id, const float *frame, bool direct, int box,
                        Clock::time_point arrival) {
    const long long ticket = srv->next_ticket++;
    Request rq;
    rq.ref = ref_id;
    rq.frame = frame;
    rq.direct = direct;
    rq.box = box;
    rq.arrival = arrival;
    rq.submitted = Clock::now();
    srv->reqs.emplace(ticket, rq);
    srv->queue.push_back(ticket);
    srv->peak_queue = std::max<long long>(srv->peak_queue, (long long)srv->queue.size());
    return ticket;
}

// Wait (at most timeout_s) for a ticket and take its record out of the table.
int take_request(glsfft_server srv, long long ticket, double timeout_s, Request *out) {
    std::unique_lock<std::mutex> lock(srv->mu);
    auto it = srv->reqs.find(ticket);
    if (it == srv->reqs.end()) return GLSFFT_ERROR_INVALID_VALUE;
    const auto deadline = Clock::now() + std::chrono::duration_cast<Clock::duration>(
                                             std::chrono::duration<double>(timeout_s));
    while (it->second.state < REQ_DONE) {
        if (srv->cv_done.wait_until(lock, deadline) == std::cv_status::timeout &&
            it->second.state < REQ_DONE)
            return GLSFFT_ERROR_TIMEOUT;
        it = srv->reqs.find(ticket);
    }
    *out = it->second;
    srv->reqs.erase(it);
    return GLSFFT_SUCCESS;
}

double seconds(Clock::time_point a, Clock::time_point b) {
    return std::chrono::duration<double>(b - a).count();
}

}  // namespace

extern "C" {

int glsfft_server_create(glsfft_context ctx, int slots, size_t hbm_budget, glsfft_server *out) {
    if (!out) return GLSFFT_ERROR_INVALID_VALUE;
    *out = nullptr;
    if (!ctx || slots < 1 || slots > 64 || hbm_budget < Arena::kAlign) return GLSFFT_ERROR_INVALID_VALUE;
    DeviceGuard g(ctx->device);
    if (!g.ok()) return GLSFFT_ERROR_CUDA;
    auto *srv = new (std::nothrow) glsfft_server_s();
    if (!srv) return GLSFFT_ERROR_OUT_OF_MEMORY;
    srv->ctx = ctx;
    srv->device = ctx->device;
    if (cudaMalloc(&srv->d_base, hbm_budget) != cudaSuccess) {
        cudaGetLastError();
        delete srv;
        return GLSFFT_ERROR_OUT_OF_MEMORY;
    }
    srv->arena.reset(hbm_budget);
    srv->slots.resize(slots);
    for (auto &s : srv->slots) {
        cudaError_t e = cudaStreamCreateWithFlags(&s.stream, cudaStreamNonBlocking);
        if (e == cudaSuccess) e = cudaEventCreate(&s.start);
        if (e == cudaSuccess) e = cudaEventCreate(&s.copied);
        if (e == cudaSuccess) e = cudaEventCreate(&s.done);
        if (e == cudaSuccess) e = cudaHostAlloc(&s.h_result, 8 * sizeof(double), cudaHostAllocMapped);
        if (e == cudaSuccess) e = cudaHostGetDevicePointer(&s.h_result_dev, s.h_result, 0);
        if (e != cudaSuccess) {
            cudaGetLastError();
            for (auto &t : srv->slots) {
                if (t.stream) cudaStreamDestroy(t.stream);
                if (t.start) cudaEventDestroy(t.start);
                if (t.copied) cudaEventDestroy(t.copied);
                if (t.done) cudaEventDestroy(t.done);
                if (t.h_result) cudaFreeHost(t.h_result);
            }
            cudaFree(srv->d_base);
            delete srv;
            return GLSFFT_ERROR_CUDA;
        }
    }
    for (int i = 0; i < kDispatchers; i++) srv->dispatchers.emplace_back(dispatcher_main, srv);
    srv->poller = std::thread(poller_main, srv);
    *out = srv;
    return GLSFFT_SUCCESS;
}

int glsfft_server_add_reference(glsfft_server srv, const float *frame, const float *window,
                                int rows, int cols, int *ref_id) {
    if (!srv || !frame || !ref_id) return GLSFFT_ERROR_INVALID_VALUE;
    int st = check_dims(rows, cols);
    if (st) return st;
    if ((reinterpret_cast<uintptr_t>(frame) & 3) || (window && (reinterpret_cast<uintptr_t>(window) & 3)))
        return GLSFFT_ERROR_MISALIGNED;
    DeviceGuard g(srv->device);
    if (!g.ok()) return GLSFFT_ERROR_CUDA;
    const size_t n = (size_t)rows * cols;
    Reference ref;
    ref.rows = rows;
    ref.cols = cols;
    ref.has_window = window != nullptr;
    {
        std::lock_guard<std::mutex> lock(srv->mu);
        ref.spec_off = srv->arena.alloc(8 * n);
        if (ref.spec_off == Arena::kFail) return GLSFFT_ERROR_BUDGET;
        if (window) {
            ref.win_off = srv->arena.alloc(4 * n);
            if (ref.win_off == Arena::kFail) {
                srv->arena.release(ref.spec_off);
                return GLSFFT_ERROR_BUDGET;
            }
        }
        srv->peak_arena = std::max(srv->peak_arena, srv->arena.in_use());
    }
    float2 *spec = reinterpret_cast<float2 *>(srv->d_base + ref.spec_off);
    float *win = window ? reinterpret_cast<float *>(srv->d_base + ref.win_off) : nullptr;
    cudaStream_t s = srv->slots[0].stream;
    cudaError_t e = cudaSuccess;
    if (window) e = cudaMemcpyAsync(win, window, 4 * n, cudaMemcpyDeviceToDevice, s);
    if (e != cudaSuccess) return cuda_status(e);
    // the reference's forward spectrum of window x frame: rows pass with the
    // window fused into the load, then the columns pass in place
    PassArgs a{};
    a.in0 = frame;
    a.out0 = spec;
    a.window = win;
    a.rows = rows;
    a.cols = cols;
    a.scale = 1.0f;
    a.tw = srv->ctx->d_tw;
    e = launch_rows(cols, win ? LD_R1W : LD_R1, ST_C2, a, 1, s);
    if (e == cudaSuccess && rows > 1) {
        PassArgs b{};
        b.in0 = spec;
        b.out0 = spec;
        b.rows = rows;
        b.cols = cols;
        b.scale = 1.0f;
        b.tw = srv->ctx->d_tw;
        e = launch_cols(rows, LD_C2, ST_C2, b, 1, s);
    }
    if (e == cudaSuccess) e = cudaStreamSynchronize(s);
    if (e != cudaSuccess) return cuda_status(e);
    std::lock_guard<std::mutex> lock(srv->mu);
    srv->refs.push_back(ref);
    *ref_id = (int)srv->refs.size() - 1;
    return GLSFFT_SUCCESS;
}

int glsfft_server_submit(glsfft_server srv, int ref_id, const float *host_frame, int box,
                         long long *ticket) {
    if (!srv || !host_frame || !ticket || box < 1) return GLSFFT_ERROR_INVALID_VALUE;
    const bool direct = srv->direct_read && frame_readable(srv, host_frame);
    std::lock_guard<std::mutex> lock(srv->mu);
    if (ref_id < 0 || ref_id >= (int)srv->refs.size()) return GLSFFT_ERROR_INVALID_VALUE;
    const Reference &ref = srv->refs[ref_id];
    if (workspace_bytes(ref.rows, ref.cols) > srv->arena.capacity()) return GLSFFT_ERROR_BUDGET;
    *ticket = submit_locked(srv, ref_id, host_frame, direct, box, Clock::now());
    srv->cv_dispatch.notify_one();
    return GLSFFT_SUCCESS;
}

int glsfft_server_wait(glsfft_server srv, long long ticket, double *result5, double *latency_s,
                       double timeout_s) {
    if (!srv) return GLSFFT_ERROR_INVALID_VALUE;
    Request rq;
    const int st = take_request(srv, ticket, timeout_s, &rq);
    if (st) return st;
    if (result5) std::memcpy(result5, rq.result, sizeof(rq.result));
    if (latency_s) *latency_s = seconds(rq.arrival, rq.done_at);
    return rq.state == REQ_DONE ? GLSFFT_SUCCESS : rq.status;
}

int glsfft_server_replay_traced(glsfft_server srv, int n, const double *offsets_s,
                                const int *ref_ids, const float *const *host_frames, int box,
                                double *latencies_s, double *results5, double *phases6) {
    if (!srv || n < 1 || !offsets_s || !ref_ids || !host_frames || !latencies_s || box < 1)
        return GLSFFT_ERROR_INVALID_VALUE;
    {
        std::lock_guard<std::mutex> lock(srv->mu);
        for (int k = 0; k < n; k++) {
            if (ref_ids[k] < 0 || ref_ids[k] >= (int)srv->refs.size() || !host_frames[k])
                return GLSFFT_ERROR_INVALID_VALUE;
            const Reference &ref = srv->refs[ref_ids[k]];
            if (workspace_bytes(ref.rows, ref.cols) > srv->arena.capacity()) return GLSFFT_ERROR_BUDGET;
        }
    }
    std::vector<long long> tickets(n);
    std::vector<char> direct(n, 0);
    if (srv->direct_read)
        for (int k = 0; k < n; k++) direct[k] = frame_readable(srv, host_frames[k]);
    const Clock::time_point t0 = Clock::now();
    for (int k = 0; k < n; k++) {
        // open-loop arrivals: latency counts from the scheduled arrival time.
        // Sleep while more than 300 us remain (a sleep can overrun by tens of
        // microseconds), then poll the clock.
        const Clock::time_point at =
            t0 + std::chrono::duration_cast<Clock::duration>(std::chrono::duration<double>(offsets_s[k]));
        for (;;) {
            const auto left = at - Clock::now();
            if (left <= Clock::duration::zero()) break;
            if (left > std::chrono::microseconds(300))
                std::this_thread::sleep_for(left - std::chrono::microseconds(250));
        }
        std::lock_guard<std::mutex> lock(srv->mu);
        tickets[k] = submit_locked(srv, ref_ids[k], host_frames[k], direct[k] != 0, box, at);
        srv->cv_dispatch.notify_one();
    }
    int status = GLSFFT_SUCCESS;
    for (int k = 0; k < n; k++) {
        Request rq;
        int st = take_request(srv, tickets[k], 60.0, &rq);
        if (!st && rq.state != REQ_DONE) st = rq.status;
        if (st && !status) status = st;
        latencies_s[k] = st ? -1.0 : seconds(rq.arrival, rq.done_at);
        if (results5) std::memcpy(results5 + 5 * (size_t)k, rq.result, sizeof(rq.result));
        if (phases6) {
            double *ph = phases6 + 6 * (size_t)k;
            ph[0] = seconds(rq.arrival, rq.submitted);   // arrival thread's lateness
            ph[1] = seconds(rq.submitted, rq.admitted);  // queued: slot / workspace / dispatcher
            ph[2] = seconds(rq.admitted, rq.launched);   // issuing the copy, launches, events
            ph[3] = seconds(rq.launched, rq.done_at);    // device work + completion polling
            ph[4] = rq.gpu_s;                            // device time, start to done event
            ph[5] = rq.copy_s;                           // of which the frame's copy
        }
    }
    return status;
}

int glsfft_server_replay(glsfft_server srv, int n, const double *offsets_s, const int *ref_ids,
                         const float *const *host_frames, int box, double *latencies_s,
                         double *results5) {
    return glsfft_server_replay_traced(srv, n, offsets_s, ref_ids, host_frames, box, latencies_s,
                                       results5, nullptr);
}

int glsfft_server_set_frame_read(glsfft_server srv, int direct) {
    if (!srv || (direct != 0 && direct != 1)) return GLSFFT_ERROR_INVALID_VALUE;
    std::lock_guard<std::mutex> lock(srv->mu);
    srv->direct_read = direct != 0;
    return GLSFFT_SUCCESS;
}

int glsfft_server_stats(glsfft_server srv, long long *out8) {
    if (!srv || !out8) return GLSFFT_ERROR_INVALID_VALUE;
    std::lock_guard<std::mutex> lock(srv->mu);
    out8[0] = srv->admitted;
    out8[1] = srv->completed;
    out8[2] = srv->failed;
    out8[3] = srv->peak_in_flight;
    out8[4] = srv->peak_queue;
    out8[5] = (long long)srv->arena.capacity();
    out8[6] = (long long)srv->peak_arena;
    out8[7] = (long long)srv->refs.size();
    return GLSFFT_SUCCESS;
}

int glsfft_server_destroy(glsfft_server srv) {
    if (!srv) return GLSFFT_ERROR_INVALID_VALUE;
    {
        std::lock_guard<std::mutex> lock(srv->mu);
        srv->stop = true;
        // requests still queued are dropped; running ones finish below
        for (long long t : srv->queue) {
            auto &rq = srv->reqs[t];
            rq.state = REQ_FAILED;
            rq.status = GLSFFT_ERROR_INVALID_VALUE;
        }
        srv->queue.clear();
    }
    srv->cv_dispatch.notify_all();
    srv->cv_poll.notify_all();
    srv->cv_done.notify_all();
    for (auto &t : srv->dispatchers)
        if (t.joinable()) t.join();
    if (srv->poller.joinable()) srv->poller.join();
    DeviceGuard g(srv->device);
    for (auto &s : srv->slots) {
        if (s.stream) {
            cudaStreamSynchronize(s.stream);
            cudaStreamDestroy(s.stream);
        }
        if (s.start) cudaEventDestroy(s.start);
        if (s.copied) cudaEventDestroy(s.copied);
        if (s.done) cudaEventDestroy(s.done);
        if (s.h_result) cudaFreeHost(s.h_result);
    }
    if (srv->d_base) cudaFree(srv->d_base);
    delete srv;
    return GLSFFT_SUCCESS;
}

}  // extern "C"
