// glsfft_internal.h -- shared declarations between the C ABI and the kernel
// translation units.  Not a public header.
#pragma once
#include <cuda_runtime.h>
#include <stddef.h>
#include <stdint.h>

namespace glsfft {

constexpr int kMaxLen = 4096;  // largest supported FFT length per dimension

// Per-pass twiddle tables: for a pass of radix R whose sub-transforms have
// length L (= span * R), entry [k][r] = e^{-2 pi i k r / L}, k < L/R, r < R,
// so a butterfly fetches its R twiddles with R/2 16-byte loads.  All tables
// live in one buffer of kTwEntries float2, table (R, L) at tw_offset(R, L).
constexpr int kTwRadixSpan = 8192;
constexpr int kTwEntries = 4 * kTwRadixSpan;
__host__ __device__ constexpr int tw_radix_index(int r) {
    return r == 2 ? 0 : r == 4 ? 1 : r == 8 ? 2 : 3;
}
__host__ __device__ constexpr int tw_offset(int r, int l) {
    return tw_radix_index(r) * kTwRadixSpan + l;
}

// load modes of the first pass
enum { LD_C2 = 0, LD_R1 = 1, LD_R1W = 2 };
// store modes of the last pass
// ST_LOGMAG_MINMAX: log(|sqrt(re^2 + im^2) + param|) stored as CV_32FC1, with
// the minMaxLoc keys of the stored values reduced into key[0] (min), key[1] (max)
enum { ST_C2 = 0, ST_RE = 1, ST_RE_ARGMAX = 2, ST_LOGMAG_MINMAX = 3 };
// per-pass flags
enum : unsigned {
    PF_CONJ_IN = 1u << 0,
    PF_CONJ_OUT = 1u << 1,
    PF_SHIFT_ROWS = 1u << 2,
    PF_SHIFT_COLS = 1u << 3,
    PF_F1_SPECTRUM = 1u << 4,
};

struct PassArgs {
    const void *in0;
    const void *in1;
    void *out0;
    void *out1;
    const float *window;
    int rows, cols;
    float scale;
    unsigned flags;
    unsigned long long *key;
    const float2 *tw;  // twiddle table of this pass's length
    size_t in_img_bytes;   // batch: byte stride between images (0 = single / in1 mode)
    size_t out_img_bytes;
    float param;       // ST_LOGMAG_MINMAX: the log-magnitude offset
    // ST_RE_ARGMAX with `result` set: the last block to finish computes the
    // phaseCorrelate centroid (box edge `box`) into result[0..4]; key[1] is
    // the block counter (zeroed, with key[0], by the POC column pass)
    double *result;
    int box;
    // with `result`: set to 1 (after a system-scope fence) once result[0..4]
    // are written, for a host that waits on it instead of the stream; or null
    unsigned long long *done_flag;
    // device status word for bounded waits (the streamed passes record
    // GLSFFT_ERROR_TIMEOUT there), or null
    int *err;
    // fault injection for tests (streamed passes): when > 0, each block
    // leaves its first tile's copy unissued and waits this many nanoseconds
    // for it, so the wait runs out
    long long stall_ns;
    // launch with programmatic dependent launch (every pass kernel begins
    // with griddepcontrol.wait): the grid may become resident before its
    // stream predecessor ends
    int pdl;
};

// Launchers (fft_rows.cu, fft_cols.cu, poc.cu).  They return cudaSuccess or
// the launch error; `images` is the grid's y extent (blockIdx.y = image).
cudaError_t launch_rows(int n, int ld, int st, const PassArgs &a, int images, cudaStream_t s);
cudaError_t launch_cols(int n, int ld, int st, const PassArgs &a, int images, cudaStream_t s);
cudaError_t launch_poc_cols(int n, const PassArgs &a, cudaStream_t s);

// The streamed column pass for 2048- and 4096-point columns (fft_stream.cu;
// cols must be true): whether it applies to these arguments (contiguous
// complex images, 16-byte aligned, the column count a multiple of the
// tile's; store mode ST_C2, or ST_LOGMAG_MINMAX over one image), and the
// launch, which gives cudaErrorNotSupported when it does not apply.
bool stream_pass_applies(int n, bool cols, const PassArgs &a, int images, int st = ST_C2);
cudaError_t launch_stream_pass(int n, bool cols, const PassArgs &a, int images, cudaStream_t s,
                               int st = ST_C2);

// A 2-D tensor map over a row-major array of 8-byte elements (width x
// height, rows `width` elements apart) with a box_w x box_h box, for TMA
// copies (batch.cpp).  GLSFFT_SUCCESS or an error status.
int make_tmap_2d(void *tmap128, const void *base, long long width, long long height, int box_w,
                 int box_h);

// Opt kernel `kern` into `bytes` of dynamic shared memory on the current
// device.  The attribute belongs to the kernel's instance on one device, so
// this runs once per (kernel, device) (thread-safe; capi.cpp).
cudaError_t smem_opt_in(const void *kern, size_t bytes);

// Twiddle tables: one device buffer of kTwEntries float2 holding the
// per-pass tables of fft_device.cuh (tw_offset).  Generated in FP64 on the
// host and rounded once to FP32.
void make_twiddle_host(float2 *dst /* kTwEntries entries */);

}  // namespace glsfft
