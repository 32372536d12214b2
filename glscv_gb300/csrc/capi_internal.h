// capi_internal.h -- the context object and host helpers shared by the C ABI
// translation units.  Not a public header.
#pragma once
#include <cuda_runtime.h>
#include <stddef.h>

#include <functional>
#include <map>

#include "glsfft.h"
#include "plan_cache.h"
#include "sched_internal.h"
#include "tc_internal.h"

struct HostPipe;  // transfer.cpp: host-buffer pipeline (streams, device slots, plans)

struct glsfft_context_s {
    int device = 0;
    float2 *d_tw = nullptr;     // twiddle tables, see make_twiddle_host
    void *ws = nullptr;         // workspace (phaseCorrelate scratch)
    size_t ws_bytes = 0;
    size_t budget = 0;          // 0 = unlimited
    double *h_result = nullptr; // pinned and mapped, 8 doubles
    double *h_result_dev = nullptr;  // its device-side address
    glsfft::TcTables tc;        // split-FP16 tensor-core form tables
    const float *surface = nullptr;  // last phaseCorrelate surface
    size_t surface_count = 0;
    // per image size (sched_key): the pass schedules the complex 2-D FFT
    // launches use; sizes not listed run schedule 0
    std::map<long long, glsfft::FftSchedule> sched;
    HostPipe *host_pipe = nullptr;  // glsfft_fft2d_host's pipeline, built on first use
    int *d_status = nullptr;  // device status word of bounded waits (glsfft_device_status)
    long long stall_ns = 0;   // glsfft_context_inject_stall (0: off)
    // the reference-arithmetic mode's twiddle tables, per line length
    std::map<int, float2 *> exact_tw;
    // glsfft_phase_correlate's three launches as a CUDA graph, replayed
    // while a call repeats the last one's buffers, shape and workspace
    struct PocGraph {
        const float *src1 = nullptr, *src2 = nullptr, *window = nullptr;
        int rows = 0, cols = 0, box = 0;
        const void *ws = nullptr;
        cudaGraphExec_t exec = nullptr;
    } poc_graph;
    cudaStream_t capture_stream = nullptr;  // private stream the graph is captured on
};

namespace glsfft {

// Sets the device for the scope of a call and restores the caller's.
class DeviceGuard {
  public:
    explicit DeviceGuard(int dev);
    ~DeviceGuard();
    bool ok() const { return ok_; }

  private:
    int prev_ = -1;
    bool ok_ = true;
};

int cuda_status(cudaError_t e);
int check_dims(int rows, int cols);  // 1..kMaxLen, powers of two
int ensure_workspace(glsfft_context ctx, size_t bytes);
int check_fft_args(const void *src, const void *dst, int rows, int cols, int flags, bool real_in);
int check_poc_args(glsfft_context ctx, const float *src1, const float *src2,
                   const float *window, int rows, int cols, int box);
int fft2d_launch(glsfft_context ctx, const void *src, void *dst, int rows, int cols, int flags,
                 bool real_in, cudaStream_t s, int count = 1);
// The reference-arithmetic transform (fft_exact.cu): `count` images src ->
// dst through tmp (count * rows * cols complex, apart from src and dst).
int fft2d_exact_launch(glsfft_context ctx, const void *src, void *dst, void *tmp, int count,
                       int rows, int cols, int flags, int algo, cudaStream_t s);

constexpr int kMaxBatch = 65535;  // grid y extent
int poc_launch(const float2 *tw, const float *src1, const float *src2, const float *window,
               int rows, int cols, int box, float2 *f1, float2 *f2, float *surface,
               unsigned long long *key, double *d_result, cudaStream_t s,
               unsigned long long *done_flag = nullptr);

void host_pipe_destroy(HostPipe *p);  // waits for its streams, frees everything

// ------------------------------------------------------------- autotuner
// The fields that identify the device a tuning was measured on.
plan_cache::Pairs device_fields(int device);
// Median of `reps` CUDA-event-timed runs of fn on stream s, after `warm`
// untimed runs.  fn returns a glsfft status; the first failure is returned.
int time_median_ms(const std::function<int()> &fn, int warm, int reps, cudaStream_t s,
                   double *ms);

// phaseCorrelate workspace: f1 | f2 (complex) | surface (float) | key | result
inline size_t poc_key_offset(int rows, int cols) {
    const size_t n = (size_t)rows * cols;
    return (20 * n + 255) / 256 * 256;
}
inline size_t poc_result_offset(int rows, int cols) { return poc_key_offset(rows, cols) + 64; }
inline size_t poc_workspace_bytes(int rows, int cols) { return poc_result_offset(rows, cols) + 64; }

}  // namespace glsfft
