// capi.cpp -- the C ABI of include/glsfft.h: argument checks, the context
// (twiddle tables + workspace) and the launch sequences of gls::fft and
// gls::phaseCorrelate.
#include "glsfft.h"

#include <atomic>
#include <chrono>
#include <cmath>
#include <cstdint>
#include <cstring>
#include <mutex>
#include <set>
#include <utility>
#include <new>
#include <vector>

#include "capi_internal.h"
#include "glsfft_internal.h"

using namespace glsfft;

// --------------------------------------------------------------- twiddles
// e^{-2 pi i k/n} (k < n, n a power of two) in FP64 from an exact quadrant /
// octant reduction, so that +-1, 0 and the pi/4 values come out exact and
// symmetric, then one rounding to FP32.
static void twiddle_d(long long k, long long n, double &re, double &im) {
    const double two_pi = 6.283185307179586476925286766559;
    k %= n;
    if (n < 4) {
        re = k == 0 ? 1.0 : -1.0;
        im = 0.0;
        return;
    }
    const long long q = (4 * k) / n;       // quadrant
    const long long r = k - q * (n / 4);   // position inside the quadrant
    double c, s;                           // cos, sin of 2 pi r / n
    if (8 * r <= n) {
        c = std::cos(two_pi * (double)r / (double)n);
        s = std::sin(two_pi * (double)r / (double)n);
    } else {
        const double a = two_pi * (double)(n / 4 - r) / (double)n;
        c = std::sin(a);
        s = std::cos(a);
    }
    for (long long i = 0; i < q; i++) {  // rotate by i^q
        const double t = c;
        c = -s;
        s = t;
    }
    re = c;   // forward sign: cos - i sin
    im = -s;
}

static float2 twiddle(long long k, long long n) {
    double re, im;
    twiddle_d(k, n, re, im);
    return make_float2((float)re, (float)im);
}

// ---------------------------------------------- tensor-core form tables
int glsfft::tc_tables_create(TcTables *t) {
    // stage-B twiddles (1024 + 4096 complex), then the two DFT operand images
    // at 1024-byte offsets
    const size_t dft_off = ((1024 + 4096) * sizeof(float2) + 1023) / 1024 * 1024;
    const size_t dft64_off = dft_off + 16384;
    const size_t bytes = dft64_off + 49152;
    std::vector<unsigned char> host(bytes, 0);
    unsigned char *p = host.data();
    float2 *tw1 = reinterpret_cast<float2 *>(p);
    float2 *tw4 = tw1 + 1024;
    // w^(k1 n2) / N1: the four-step twiddle with the stage-C scale folded in
    // (a power of two, so the division is exact)
    for (int k1 = 0; k1 < 32; k1++)
        for (int n2 = 0; n2 < 32; n2++) {
            const float2 w = twiddle((long long)k1 * n2, 1024);
            tw1[k1 * 32 + n2] = make_float2(w.x / 32.0f, w.y / 32.0f);
        }
    for (int k1 = 0; k1 < 64; k1++)
        for (int n2 = 0; n2 < 64; n2++) {
            const float2 w = twiddle((long long)k1 * n2, 4096);
            tw4[k1 * 64 + n2] = make_float2(w.x / 64.0f, w.y / 64.0f);
        }
    double cs[64][2];
    for (int n1 = 32; n1 <= 64; n1 *= 2) {
        for (int m = 0; m < n1; m++) {
            double re, im;  // e^{-2 pi i m / n1} = cos - i sin
            twiddle_d(m, n1, re, im);
            cs[m][0] = re;
            cs[m][1] = -im;
        }
        tc5_dft_image(n1, cs, p + (n1 == 32 ? dft_off : dft64_off));
    }
    void *d = nullptr;
    cudaError_t e = cudaMalloc(&d, bytes);
    if (e == cudaSuccess) e = cudaMemcpy(d, host.data(), bytes, cudaMemcpyHostToDevice);
    if (e != cudaSuccess) {
        cudaGetLastError();
        if (d) cudaFree(d);
        return cuda_status(e);
    }
    unsigned char *b = static_cast<unsigned char *>(d);
    t->block = d;
    t->tw1024 = reinterpret_cast<float2 *>(b);
    t->tw4096 = reinterpret_cast<float2 *>(b) + 1024;
    t->dft32_sw = b + dft_off;
    t->dft64_sw = b + dft64_off;
    return GLSFFT_SUCCESS;
}

void glsfft::tc_tables_destroy(TcTables *t) {
    if (t->block) cudaFree(t->block);
    *t = TcTables{};
}

// Per-pass tables (see tw_offset), for every radix R and every length
// R <= L <= kTwRadixSpan / 2: row k < L/R of table (R, L) holds
// w^r = e^{-2 pi i k r / L} for 1 <= r < R/2 in slot r and w^(R/2) in slot 0
// (the line engine derives w^(R/2+r) = w^(R/2) w^r); for R = 2 slot 0 holds w^1.
void glsfft::make_twiddle_host(float2 *dst) {
    for (int i = 0; i < kTwEntries; i++) dst[i] = make_float2(0.f, 0.f);
    for (int radix = 2; radix <= 16; radix <<= 1)
        for (int l = radix; l <= kTwRadixSpan / 2; l <<= 1)
            for (int k = 0; k < l / radix; k++) {
                float2 *row = dst + tw_offset(radix, l) + k * radix;
                if (radix == 2) {
                    row[0] = twiddle(k, l);
                    continue;
                }
                row[0] = twiddle((long long)k * (radix / 2), l);
                for (int r = 1; r < radix / 2; r++) row[r] = twiddle((long long)k * r, l);
            }
}

// ---------------------------------------------------------------- helpers
namespace {

inline bool is_pow2(int x) { return x > 0 && (x & (x - 1)) == 0; }

inline bool aligned(const void *p, size_t a) { return (reinterpret_cast<uintptr_t>(p) % a) == 0; }

}  // namespace

int glsfft::check_dims(int rows, int cols) {
    if (rows < 1 || cols < 1 || rows > kMaxLen || cols > kMaxLen) return GLSFFT_ERROR_SIZE;
    if (!is_pow2(rows) || !is_pow2(cols)) return GLSFFT_ERROR_NOT_POW2;
    return GLSFFT_SUCCESS;
}

int glsfft::cuda_status(cudaError_t e) {
    if (e == cudaSuccess) return GLSFFT_SUCCESS;
    if (e == cudaErrorMemoryAllocation) return GLSFFT_ERROR_OUT_OF_MEMORY;
    return GLSFFT_ERROR_CUDA;
}

DeviceGuard::DeviceGuard(int dev) {
    if (cudaGetDevice(&prev_) != cudaSuccess) prev_ = -1;
    if (prev_ != dev) ok_ = cudaSetDevice(dev) == cudaSuccess;
}
DeviceGuard::~DeviceGuard() {
    int cur = -1;
    if (prev_ >= 0 && cudaGetDevice(&cur) == cudaSuccess && cur != prev_) cudaSetDevice(prev_);
}

cudaError_t glsfft::smem_opt_in(const void *kern, size_t bytes) {
    static std::mutex mu;
    static std::set<std::pair<const void *, int>> done;
    int dev = 0;
    cudaError_t e = cudaGetDevice(&dev);
    if (e != cudaSuccess) return e;
    std::lock_guard<std::mutex> lock(mu);
    if (done.count({kern, dev})) return cudaSuccess;
    e = cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)bytes);
    if (e == cudaSuccess) done.insert({kern, dev});
    return e;
}

int glsfft::ensure_workspace(glsfft_context ctx, size_t bytes) {
    // every user of the workspace overwrites (or frees) the last
    // phaseCorrelate's surface; the phaseCorrelate calls record theirs after
    ctx->surface = nullptr;
    ctx->surface_count = 0;
    if (bytes <= ctx->ws_bytes) return GLSFFT_SUCCESS;
    if (ctx->budget && bytes > ctx->budget) return GLSFFT_ERROR_BUDGET;
    if (ctx->ws) {
        cudaError_t e = cudaFree(ctx->ws);
        ctx->ws = nullptr;
        ctx->ws_bytes = 0;
        if (e != cudaSuccess) return cuda_status(e);
    }
    void *p = nullptr;
    cudaError_t e = cudaMalloc(&p, bytes);
    if (e != cudaSuccess) {
        cudaGetLastError();
        return GLSFFT_ERROR_OUT_OF_MEMORY;
    }
    ctx->ws = p;
    ctx->ws_bytes = bytes;
    return GLSFFT_SUCCESS;
}

// The two passes of gls::fft over `count` back-to-back images (one launch
// per pass for the whole batch).  `real_in`: src is CV_32FC1 (promote).
// Both launches use programmatic dependent launch: the column pass is
// resident and waiting while the row pass drains, and the row pass of the
// next call on the stream likewise behind this call's column pass.
int glsfft::fft2d_launch(glsfft_context ctx, const void *src, void *dst, int rows, int cols,
                         int flags, bool real_in, cudaStream_t s, int count) {
    const bool inv = flags & GLSFFT_INVERSE, scale = flags & GLSFFT_SCALE,
               shift = flags & GLSFFT_SHIFT;
    const bool do_rows = cols > 1 || rows == 1 || real_in;
    const bool do_cols = rows > 1;
    const size_t px = (size_t)rows * cols;
    const FftSchedule sc = schedule_for(ctx->sched, rows, cols);
    if (do_rows) {
        PassArgs a{};
        a.in0 = src;
        a.out0 = dst;
        a.rows = rows;
        a.cols = cols;
        a.scale = scale ? 1.0f / (float)cols : 1.0f;
        a.flags = (inv ? PF_CONJ_IN : 0u) | (inv && !do_cols ? PF_CONJ_OUT : 0u) |
                  (shift ? PF_SHIFT_COLS : 0u);
        a.tw = ctx->d_tw;
        a.err = ctx->d_status;
        a.stall_ns = ctx->stall_ns;
        a.in_img_bytes = px * (real_in ? sizeof(float) : sizeof(float2));
        a.out_img_bytes = px * sizeof(float2);
        a.pdl = 1;
        cudaError_t e = real_in ? launch_rows(cols, LD_R1, ST_C2, a, count, s)
                                : launch_rows_sched(cols, sc.row, a, count, s);
        if (e != cudaSuccess) return cuda_status(e);
    }
    if (do_cols) {
        PassArgs a{};
        a.in0 = do_rows ? dst : src;
        a.out0 = dst;
        a.rows = rows;
        a.cols = cols;
        a.scale = scale ? 1.0f / (float)rows : 1.0f;
        a.flags = (inv && !do_rows ? PF_CONJ_IN : 0u) | (inv ? PF_CONJ_OUT : 0u) |
                  (shift ? PF_SHIFT_ROWS : 0u);
        a.tw = ctx->d_tw;
        a.err = ctx->d_status;
        a.stall_ns = ctx->stall_ns;
        a.in_img_bytes = a.out_img_bytes = px * sizeof(float2);
        a.pdl = 1;
        cudaError_t e = launch_cols_sched(rows, sc.col, a, count, s);
        if (e != cudaSuccess) return cuda_status(e);
    }
    return GLSFFT_SUCCESS;
}

// phaseCorrelate launch sequence on caller-provided scratch:
// f1, f2: rows*cols complex each; surface: rows*cols floats; key: 8 bytes.
int glsfft::poc_launch(const float2 *tw, const float *src1, const float *src2,
                       const float *window, int rows, int cols, int box, float2 *f1, float2 *f2,
                       float *surface, unsigned long long *key, double *d_result,
                       cudaStream_t s, unsigned long long *done_flag) {
    // three launches: rows of both images; fused POC columns (which also
    // zero the argmax key and block counter); inverse rows with the argmax
    // and, in the last block, the centroid.  All three use programmatic
    // dependent launch, so each grid is resident and waiting when its
    // predecessor (the previous call's last pass, for the first) ends.
    PassArgs a{};
    a.in0 = src1;
    a.in1 = src2;
    a.out0 = f1;
    a.out1 = f2;
    a.window = window;
    a.rows = rows;
    a.cols = cols;
    a.scale = 1.0f;
    a.tw = tw;
    a.pdl = 1;
    cudaError_t e = launch_rows(cols, window ? LD_R1W : LD_R1, ST_C2, a, 2, s);
    if (e != cudaSuccess) return cuda_status(e);

    PassArgs b{};
    b.in0 = f1;
    b.in1 = f2;
    b.out0 = f1;
    b.rows = rows;
    b.cols = cols;
    b.scale = 1.0f;
    b.key = key;
    b.tw = tw;
    b.pdl = 1;
    e = launch_poc_cols(rows, b, s);
    if (e != cudaSuccess) return cuda_status(e);

    PassArgs c{};
    c.in0 = f1;
    c.out0 = surface;
    c.rows = rows;
    c.cols = cols;
    c.scale = 1.0f;
    c.flags = PF_SHIFT_ROWS | PF_SHIFT_COLS;
    c.key = key;
    c.tw = tw;
    c.result = d_result;
    c.box = box;
    c.done_flag = done_flag;
    c.pdl = 1;
    e = launch_rows(cols, LD_C2, ST_RE_ARGMAX, c, 1, s);
    return cuda_status(e);
}

int glsfft::check_poc_args(glsfft_context ctx, const float *src1, const float *src2,
                           const float *window, int rows, int cols, int box) {
    if (!src1 || !src2) return GLSFFT_ERROR_INVALID_VALUE;
    int st = check_dims(rows, cols);
    if (st) return st;
    if (box < 1) return GLSFFT_ERROR_INVALID_VALUE;
    if (!aligned(src1, 4) || !aligned(src2, 4) || (window && !aligned(window, 4)))
        return GLSFFT_ERROR_MISALIGNED;
    if (!ctx) return GLSFFT_ERROR_INVALID_VALUE;
    return GLSFFT_SUCCESS;
}

int glsfft::check_fft_args(const void *src, const void *dst, int rows, int cols, int flags,
                           bool real_in) {
    if (!src || !dst) return GLSFFT_ERROR_INVALID_VALUE;
    if (flags & ~(GLSFFT_INVERSE | GLSFFT_SCALE | GLSFFT_SHIFT)) return GLSFFT_ERROR_INVALID_VALUE;
    int st = check_dims(rows, cols);
    if (st) return st;
    if (!aligned(src, real_in ? 4 : 8) || !aligned(dst, 8)) return GLSFFT_ERROR_MISALIGNED;
    return GLSFFT_SUCCESS;
}

// ------------------------------------------------------------------ C ABI
extern "C" {

const char *glsfft_status_string(int status) {
    switch (status) {
    case GLSFFT_SUCCESS: return "success";
    case GLSFFT_ERROR_INVALID_VALUE: return "invalid value (NULL pointer or handle, unknown flag, bad box)";
    case GLSFFT_ERROR_NOT_POW2: return "size is not a power of two";
    case GLSFFT_ERROR_SIZE: return "size outside [1, GLSFFT_MAX_LEN]";
    case GLSFFT_ERROR_MISALIGNED: return "pointer not aligned to its element size";
    case GLSFFT_ERROR_CUDA: return "CUDA runtime error";
    case GLSFFT_ERROR_OUT_OF_MEMORY: return "device memory allocation failed";
    case GLSFFT_ERROR_BUDGET: return "workspace would exceed the context's HBM budget";
    case GLSFFT_ERROR_TIMEOUT: return "bounded device-side wait expired";
    case GLSFFT_ERROR_SHAPE: return "inputs have different shapes";
    case GLSFFT_ERROR_NOALLOC_LIMIT:
        return "rows*cols exceeds the static scratch of glsfft_phase_correlate_noalloc "
               "(GLSFFT_NOALLOC_MAX_PIXELS)";
    case GLSFFT_ERROR_IO: return "the plan cache file could not be written";
    default: return "unknown status";
    }
}

int glsfft_version(void) { return 200; }

int glsfft_context_create(glsfft_context *out, int device) {
    if (!out) return GLSFFT_ERROR_INVALID_VALUE;
    *out = nullptr;
    int ndev = 0;
    cudaError_t e = cudaGetDeviceCount(&ndev);
    if (e != cudaSuccess) {
        cudaGetLastError();
        return GLSFFT_ERROR_CUDA;
    }
    if (device < 0 || device >= ndev) return GLSFFT_ERROR_INVALID_VALUE;
    DeviceGuard g(device);
    if (!g.ok()) return GLSFFT_ERROR_CUDA;
    auto *ctx = new (std::nothrow) glsfft_context_s();
    if (!ctx) return GLSFFT_ERROR_OUT_OF_MEMORY;
    ctx->device = device;
    std::vector<float2> tw((size_t)kTwEntries);
    make_twiddle_host(tw.data());
    e = cudaMalloc(&ctx->d_tw, sizeof(float2) * tw.size());
    if (e == cudaSuccess)
        e = cudaMemcpy(ctx->d_tw, tw.data(), sizeof(float2) * tw.size(), cudaMemcpyHostToDevice);
    if (e == cudaSuccess) e = cudaHostAlloc(&ctx->h_result, 8 * sizeof(double), cudaHostAllocMapped);
    if (e == cudaSuccess) e = cudaHostGetDevicePointer(&ctx->h_result_dev, ctx->h_result, 0);
    if (e == cudaSuccess) e = cudaMalloc(&ctx->d_status, sizeof(int));
    if (e == cudaSuccess) e = cudaMemset(ctx->d_status, 0, sizeof(int));
    int st = cuda_status(e);
    if (!st) st = tc_tables_create(&ctx->tc);
    if (st) {
        cudaGetLastError();
        if (ctx->d_tw) cudaFree(ctx->d_tw);
        if (ctx->h_result) cudaFreeHost(ctx->h_result);
        if (ctx->d_status) cudaFree(ctx->d_status);
        delete ctx;
        return st;
    }
    *out = ctx;
    return GLSFFT_SUCCESS;
}

int glsfft_context_destroy(glsfft_context ctx) {
    if (!ctx) return GLSFFT_ERROR_INVALID_VALUE;
    DeviceGuard g(ctx->device);
    host_pipe_destroy(ctx->host_pipe);  // its batch plans use the context
    if (ctx->poc_graph.exec) cudaGraphExecDestroy(ctx->poc_graph.exec);
    if (ctx->capture_stream) cudaStreamDestroy(ctx->capture_stream);
    if (ctx->ws) cudaFree(ctx->ws);
    if (ctx->d_tw) cudaFree(ctx->d_tw);
    if (ctx->h_result) cudaFreeHost(ctx->h_result);
    if (ctx->d_status) cudaFree(ctx->d_status);
    for (auto &t : ctx->exact_tw) cudaFree(t.second);
    tc_tables_destroy(&ctx->tc);
    delete ctx;
    return GLSFFT_SUCCESS;
}

int glsfft_context_inject_stall(glsfft_context ctx, long long wait_limit_ns) {
    if (!ctx || wait_limit_ns < 0) return GLSFFT_ERROR_INVALID_VALUE;
    ctx->stall_ns = wait_limit_ns;
    return GLSFFT_SUCCESS;
}

int glsfft_device_status(glsfft_context ctx, int clear) {
    if (!ctx) return GLSFFT_ERROR_INVALID_VALUE;
    DeviceGuard g(ctx->device);
    if (!g.ok()) return GLSFFT_ERROR_CUDA;
    int v = 0;
    // every stream of the device, blocking or not, has finished its work
    cudaError_t e = cudaDeviceSynchronize();
    if (e == cudaSuccess) e = cudaMemcpy(&v, ctx->d_status, sizeof(int), cudaMemcpyDeviceToHost);
    if (e == cudaSuccess && clear && v) e = cudaMemset(ctx->d_status, 0, sizeof(int));
    if (e != cudaSuccess) return cuda_status(e);
    return v;
}

int glsfft_fft2d_tc(glsfft_context ctx, const void *src, void *dst, int count, int rows,
                    int cols, int flags, void *stream) {
    int st = check_fft_args(src, dst, rows, cols, flags, false);
    if (st) return st;
    if (count < 1 || count > kMaxBatch) return GLSFFT_ERROR_INVALID_VALUE;
    if ((rows != 1024 && rows != 4096) || (cols != 1024 && cols != 4096)) return GLSFFT_ERROR_SIZE;
    if (!ctx) return GLSFFT_ERROR_INVALID_VALUE;
    DeviceGuard g(ctx->device);
    if (!g.ok()) return GLSFFT_ERROR_CUDA;
    const bool inv = flags & GLSFFT_INVERSE, scale = flags & GLSFFT_SCALE,
               shift = flags & GLSFFT_SHIFT;
    const size_t bytes = (size_t)rows * cols * sizeof(float2);
    cudaStream_t s = (cudaStream_t)stream;
    PassArgs a{};
    a.in0 = src;
    a.out0 = dst;
    a.rows = rows;
    a.cols = cols;
    a.scale = scale ? 1.0f / (float)cols : 1.0f;
    a.flags = (inv ? PF_CONJ_IN : 0u) | (shift ? PF_SHIFT_COLS : 0u);
    a.in_img_bytes = a.out_img_bytes = bytes;
    a.err = ctx->d_status;  // bounded waits record GLSFFT_ERROR_TIMEOUT here
    cudaError_t e = launch_tc_lines(cols, true, a, ctx->tc, count, s);
    if (e != cudaSuccess) return cuda_status(e);
    PassArgs b{};
    b.in0 = dst;
    b.out0 = dst;
    b.rows = rows;
    b.cols = cols;
    b.scale = scale ? 1.0f / (float)rows : 1.0f;
    b.flags = (inv ? PF_CONJ_OUT : 0u) | (shift ? PF_SHIFT_ROWS : 0u);
    b.in_img_bytes = b.out_img_bytes = bytes;
    b.err = ctx->d_status;
    return cuda_status(launch_tc_lines(rows, false, b, ctx->tc, count, s));
}

int glsfft_context_set_budget(glsfft_context ctx, size_t bytes) {
    if (!ctx) return GLSFFT_ERROR_INVALID_VALUE;
    ctx->budget = bytes;
    return GLSFFT_SUCCESS;
}

int glsfft_context_workspace(glsfft_context ctx, size_t *bytes) {
    if (!ctx || !bytes) return GLSFFT_ERROR_INVALID_VALUE;
    *bytes = ctx->ws_bytes;
    return GLSFFT_SUCCESS;
}

int glsfft_fft2d_c2c(glsfft_context ctx, const void *src, void *dst, int rows, int cols,
                     int flags, void *stream) {
    int st = check_fft_args(src, dst, rows, cols, flags, false);
    if (st) return st;
    if (!ctx) return GLSFFT_ERROR_INVALID_VALUE;
    DeviceGuard g(ctx->device);
    if (!g.ok()) return GLSFFT_ERROR_CUDA;
    return fft2d_launch(ctx, src, dst, rows, cols, flags, false, (cudaStream_t)stream);
}

int glsfft_fft2d_r2c_promote(glsfft_context ctx, const float *src, void *dst, int rows,
                             int cols, int flags, void *stream) {
    int st = check_fft_args(src, dst, rows, cols, flags, true);
    if (st) return st;
    if (!ctx) return GLSFFT_ERROR_INVALID_VALUE;
    DeviceGuard g(ctx->device);
    if (!g.ok()) return GLSFFT_ERROR_CUDA;
    return fft2d_launch(ctx, src, dst, rows, cols, flags, true, (cudaStream_t)stream);
}

static int one_pass(glsfft_context ctx, const void *src, void *dst, int count, int rows,
                    int cols, int flags, bool along_rows, cudaStream_t s) {
    int st = check_fft_args(src, dst, rows, cols, flags, false);
    if (st) return st;
    if (count < 1 || count > kMaxBatch) return GLSFFT_ERROR_INVALID_VALUE;
    if (!ctx) return GLSFFT_ERROR_INVALID_VALUE;
    DeviceGuard g(ctx->device);
    if (!g.ok()) return GLSFFT_ERROR_CUDA;
    const bool inv = flags & GLSFFT_INVERSE;
    const int n = along_rows ? cols : rows;
    PassArgs a{};
    a.in0 = src;
    a.out0 = dst;
    a.rows = rows;
    a.cols = cols;
    a.scale = (flags & GLSFFT_SCALE) ? 1.0f / (float)n : 1.0f;
    a.flags = (inv ? PF_CONJ_IN | PF_CONJ_OUT : 0u) |
              ((flags & GLSFFT_SHIFT) ? (along_rows ? PF_SHIFT_COLS : PF_SHIFT_ROWS) : 0u);
    a.tw = ctx->d_tw;
    a.err = ctx->d_status;
        a.stall_ns = ctx->stall_ns;
    a.in_img_bytes = a.out_img_bytes = (size_t)rows * cols * sizeof(float2);
    const FftSchedule sc = schedule_for(ctx->sched, rows, cols);
    cudaError_t e = along_rows ? launch_rows_sched(n, sc.row, a, count, s)
                               : launch_cols_sched(n, sc.col, a, count, s);
    return cuda_status(e);
}

int glsfft_fft_rows(glsfft_context ctx, const void *src, void *dst, int count, int rows,
                    int cols, int flags, void *stream) {
    return one_pass(ctx, src, dst, count, rows, cols, flags, true, (cudaStream_t)stream);
}

int glsfft_fft_cols(glsfft_context ctx, const void *src, void *dst, int count, int rows,
                    int cols, int flags, void *stream) {
    return one_pass(ctx, src, dst, count, rows, cols, flags, false, (cudaStream_t)stream);
}

int glsfft_fft2d_batched(glsfft_context ctx, const void *src, void *dst, int count, int rows,
                         int cols, int flags, void *stream) {
    int st = check_fft_args(src, dst, rows, cols, flags, false);
    if (st) return st;
    if (count < 1 || count > kMaxBatch) return GLSFFT_ERROR_INVALID_VALUE;
    if (!ctx) return GLSFFT_ERROR_INVALID_VALUE;
    DeviceGuard g(ctx->device);
    if (!g.ok()) return GLSFFT_ERROR_CUDA;
    return fft2d_launch(ctx, src, dst, rows, cols, flags, false, (cudaStream_t)stream, count);
}

int glsfft_phase_correlate_async(glsfft_context ctx, const float *src1, const float *src2,
                                 const float *window, int rows, int cols, int box,
                                 double *d_result, void *stream) {
    int st = check_poc_args(ctx, src1, src2, window, rows, cols, box);
    if (st) return st;
    if (!d_result) return GLSFFT_ERROR_INVALID_VALUE;
    if (!aligned(d_result, 8)) return GLSFFT_ERROR_MISALIGNED;
    DeviceGuard g(ctx->device);
    if (!g.ok()) return GLSFFT_ERROR_CUDA;
    const size_t n = (size_t)rows * cols;
    const size_t bytes = poc_workspace_bytes(rows, cols);
    st = ensure_workspace(ctx, bytes);
    if (st) return st;
    char *ws = static_cast<char *>(ctx->ws);
    float2 *f1 = reinterpret_cast<float2 *>(ws);
    float2 *f2 = f1 + n;
    float *surface = reinterpret_cast<float *>(f2 + n);
    auto *key = reinterpret_cast<unsigned long long *>(ws + poc_key_offset(rows, cols));
    ctx->surface = surface;
    ctx->surface_count = n;
    return poc_launch(ctx->d_tw, src1, src2, window, rows, cols, box, f1, f2, surface, key,
                      d_result, (cudaStream_t)stream);
}

// The synchronous call's three launches into the context's mapped result:
// a replay of the cached graph when the call repeats the last one's
// buffers, shape and workspace (one graph launch instead of three kernel
// launches), else the launches captured into a new graph on the context's
// private stream and that graph launched; if the capture is refused, the
// launches themselves.
static int poc_sync_launch(glsfft_context ctx, const float *src1, const float *src2,
                           const float *window, int rows, int cols, int box, cudaStream_t s) {
    const size_t n = (size_t)rows * cols;
    int st = ensure_workspace(ctx, poc_workspace_bytes(rows, cols));
    if (st) return st;
    // the completion flag in the mapped result buffer (double 7, past the
    // five result values)
    unsigned long long *flag = reinterpret_cast<unsigned long long *>(ctx->h_result_dev + 7);
    char *ws = static_cast<char *>(ctx->ws);
    float2 *f1 = reinterpret_cast<float2 *>(ws);
    float2 *f2 = f1 + n;
    float *surface = reinterpret_cast<float *>(f2 + n);
    auto *key = reinterpret_cast<unsigned long long *>(ws + poc_key_offset(rows, cols));
    ctx->surface = surface;
    ctx->surface_count = n;
    auto &pg = ctx->poc_graph;
    auto same = [&] {
        return pg.exec && pg.src1 == src1 && pg.src2 == src2 && pg.window == window &&
               pg.rows == rows && pg.cols == cols && pg.box == box && pg.ws == ctx->ws;
    };
    if (!same()) {
        if (pg.exec) cudaGraphExecDestroy(pg.exec);
        pg = glsfft_context_s::PocGraph{};
        if (!ctx->capture_stream &&
            cudaStreamCreateWithFlags(&ctx->capture_stream, cudaStreamNonBlocking) != cudaSuccess)
            ctx->capture_stream = nullptr;
        if (ctx->capture_stream &&
            cudaStreamBeginCapture(ctx->capture_stream, cudaStreamCaptureModeThreadLocal) ==
                cudaSuccess) {
            cudaGraph_t graph = nullptr;
            st = poc_launch(ctx->d_tw, src1, src2, window, rows, cols, box, f1, f2, surface, key,
                            ctx->h_result_dev, ctx->capture_stream, flag);
            const cudaError_t e = cudaStreamEndCapture(ctx->capture_stream, &graph);
            cudaGraphExec_t exec = nullptr;
            if (!st && e == cudaSuccess && graph && cudaGraphInstantiate(&exec, graph, 0) == cudaSuccess)
                pg = {src1, src2, window, rows, cols, box, ctx->ws, exec};
            if (graph) cudaGraphDestroy(graph);
        }
        cudaGetLastError();  // a refused capture leaves no error behind
    }
    if (same()) return cuda_status(cudaGraphLaunch(pg.exec, s));
    return poc_launch(ctx->d_tw, src1, src2, window, rows, cols, box, f1, f2, surface, key,
                      ctx->h_result_dev, s, flag);
}

int glsfft_phase_correlate(glsfft_context ctx, const float *src1, const float *src2,
                           const float *window, int rows, int cols, int box, double *dx,
                           double *dy, double *response, void *stream) {
    if (!dx || !dy) return GLSFFT_ERROR_INVALID_VALUE;
    int st = check_poc_args(ctx, src1, src2, window, rows, cols, box);
    if (st) return st;
    DeviceGuard g(ctx->device);
    if (!g.ok()) return GLSFFT_ERROR_CUDA;
    // The last block writes the result straight into the context's mapped
    // pinned buffer and then sets the completion flag there: the host spins
    // on the flag (no copy back; it returns as soon as the result is out,
    // without waiting for the kernel's exit to reach the stream), asking the
    // stream every 20 us whether it ended or failed first -- then the
    // stream's own synchronisation reports it.
    volatile unsigned long long *flag = reinterpret_cast<unsigned long long *>(ctx->h_result + 7);
    *flag = 0ull;
    st = poc_sync_launch(ctx, src1, src2, window, rows, cols, box, (cudaStream_t)stream);
    if (st) return st;
    bool seen = false;
    auto next_query = std::chrono::steady_clock::now() + std::chrono::microseconds(20);
    for (;;) {
        if (*flag) {
            seen = true;
            break;
        }
        const auto now = std::chrono::steady_clock::now();
        if (now >= next_query) {
            if (cudaStreamQuery((cudaStream_t)stream) != cudaErrorNotReady) break;
            next_query = now + std::chrono::microseconds(20);
        }
    }
    if (seen) {
        std::atomic_thread_fence(std::memory_order_acquire);  // the results after the flag
    } else {
        cudaError_t e = cudaStreamSynchronize((cudaStream_t)stream);
        if (e != cudaSuccess) return cuda_status(e);
    }
    *dx = ctx->h_result[0];
    *dy = ctx->h_result[1];
    if (response) *response = ctx->h_result[2];
    return GLSFFT_SUCCESS;
}

int glsfft_phase_correlate_surface(glsfft_context ctx, float *dst, size_t count, void *stream) {
    if (!ctx || !dst) return GLSFFT_ERROR_INVALID_VALUE;
    if (!ctx->surface || count != ctx->surface_count) return GLSFFT_ERROR_SHAPE;
    DeviceGuard g(ctx->device);
    if (!g.ok()) return GLSFFT_ERROR_CUDA;
    return cuda_status(cudaMemcpyAsync(dst, ctx->surface, count * sizeof(float),
                                       cudaMemcpyDeviceToDevice, (cudaStream_t)stream));
}

}  // extern "C"
