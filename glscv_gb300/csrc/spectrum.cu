// spectrum.cu -- the spectrum operations next to the FFT (mulSpectrums,
// mulSpectrumsPhaseOnly, magSpectrums, logMagSpectrums), gls::minMaxLoc,
// gls::normalize(NORM_MINMAX) and glsCam's FFT display pipeline, on device
// buffers.  The element kernels are HBM-bound streams (grid-stride, one
// complex or float per thread per step); minMaxLoc is a key reduction with one
// atomic per block; normalize reads the min / max keys on the device, so the
// display pipeline needs no host round trip.
//
// Reference (paths inside glsCV):
//   mulSpectrums / PhaseOnly / magSpectrums / logMagSpectrums
//                          glsCV/glsBasicOperation.cpp:320-351, shaders :92-212
//   minMaxLoc              glsCV/glsMinMaxLoc.cpp:65-119, :149-200
//   normalize NORM_MINMAX  glsCV/glsNormalize.cpp:52-68
//   glsCam FFT view        glsCam/glsCam.cpp:196-203
#include <cuda_runtime.h>

#include <cstdint>

#include "capi_internal.h"
#include "fft_device.cuh"
#include "glsfft.h"
#include "glsfft_internal.h"
#include "pdl.cuh"
#include "spectrum_device.cuh"

using namespace glsfft;

namespace {

constexpr int kThreads = 256;

// Blocks for n elements: one wave of the kernel's resident blocks at most
// (grid-stride beyond).  A grid of more blocks than fit at once would run a
// partial second wave at a fraction of the occupancy.
template <class Kernel>
int grid_for(Kernel kern, size_t n) {
    int dev = 0, sms = 0, per_sm = 0;
    cudaGetDevice(&dev);
    cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
    if (cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, kern, kThreads, 0) != cudaSuccess) {
        cudaGetLastError();
        per_sm = 1;
    }
    if (sms <= 0) sms = 1;
    if (per_sm <= 0) per_sm = 1;
    const size_t want = (n + kThreads - 1) / kThreads;
    const size_t cap = (size_t)sms * per_sm;
    return (int)(want < cap ? (want ? want : 1) : cap);
}

// The element kernels move 16 bytes per load and store (two complex or four
// float values per step; a scalar loop covers a misaligned or odd tail) and
// issue the loads of two steps (four for the float-input kernels) before
// using them, so each thread keeps several loads in flight and a grid of
// eight resident blocks per SM streams at HBM rate.
__device__ __forceinline__ bool al16(const void *p) {
    return (reinterpret_cast<uintptr_t>(p) & 15) == 0;
}

// d may equal a or b (in place): each element is read, then written, by one thread
template <int OP>  // 0: a*b, 1: a*conj(b), 2: phase only
__device__ __forceinline__ float2 spec_binary_op(float2 x, float2 y) {
    return OP == 0 ? spec_mul<false>(x, y) : OP == 1 ? spec_mul<true>(x, y) : spec_poc(x, y);
}
template <int OP>
__global__ void __launch_bounds__(kThreads) spec_binary_kernel(const float2 *a, const float2 *b,
                                                              float2 *d, size_t n) {
    const size_t tid = blockIdx.x * (size_t)blockDim.x + threadIdx.x;
    const size_t stride = (size_t)gridDim.x * blockDim.x;
    size_t done = 0;
    if (al16(a) && al16(b) && al16(d)) {
        const size_t nv = n / 2;
        const float4 *a4 = reinterpret_cast<const float4 *>(a);
        const float4 *b4 = reinterpret_cast<const float4 *>(b);
        float4 *d4 = reinterpret_cast<float4 *>(d);
        auto step = [&](const float4 x, const float4 y) {
            const float2 r0 = spec_binary_op<OP>(make_float2(x.x, x.y), make_float2(y.x, y.y));
            const float2 r1 = spec_binary_op<OP>(make_float2(x.z, x.w), make_float2(y.z, y.w));
            return make_float4(r0.x, r0.y, r1.x, r1.y);
        };
        size_t i = tid;
        for (; i + stride < nv; i += 2 * stride) {  // both steps' loads in flight
            const float4 x0 = a4[i], y0 = b4[i], x1 = a4[i + stride], y1 = b4[i + stride];
            d4[i] = step(x0, y0);
            d4[i + stride] = step(x1, y1);
        }
        if (i < nv) d4[i] = step(a4[i], b4[i]);
        done = nv * 2;
    }
    for (size_t i = done + tid; i < n; i += stride) d[i] = spec_binary_op<OP>(a[i], b[i]);
}

// magnitude or log-magnitude; with KEYS, also the minMaxLoc keys of the
// output (row-major index = element index)
template <bool LOG>
__device__ __forceinline__ float mag_op(float2 x, float offset) {
    return LOG ? spec_log_mag(x, offset) : spec_mag(x);
}
__device__ __forceinline__ void keys_add(float v, size_t i, unsigned long long &kmin,
                                         unsigned long long &kmax) {
    const unsigned long long k0 = min_key(v, (unsigned)i), k1 = max_key(v, (unsigned)i);
    kmin = k0 > kmin ? k0 : kmin;
    kmax = k1 > kmax ? k1 : kmax;
}
template <bool LOG, bool KEYS>
__global__ void __launch_bounds__(kThreads) spec_mag_kernel(const float2 *__restrict__ a,
                                                           float *__restrict__ d, size_t n,
                                                           float offset,
                                                           unsigned long long *keys) {
    __shared__ unsigned long long red[2 * (kThreads / 32)];
    unsigned long long kmin = 0, kmax = 0;
    const size_t tid = blockIdx.x * (size_t)blockDim.x + threadIdx.x;
    const size_t stride = (size_t)gridDim.x * blockDim.x;
    size_t done = 0;
    if (al16(a) && al16(d)) {  // four complex in, four float out per step
        const size_t nv = n / 4;
        const float4 *a4 = reinterpret_cast<const float4 *>(a);
        float4 *d4 = reinterpret_cast<float4 *>(d);
        auto step = [&](size_t i, const float4 p, const float4 q) {
            const float4 r = make_float4(mag_op<LOG>(make_float2(p.x, p.y), offset),
                                         mag_op<LOG>(make_float2(p.z, p.w), offset),
                                         mag_op<LOG>(make_float2(q.x, q.y), offset),
                                         mag_op<LOG>(make_float2(q.z, q.w), offset));
            d4[i] = r;
            if constexpr (KEYS) {
                keys_add(r.x, 4 * i, kmin, kmax);
                keys_add(r.y, 4 * i + 1, kmin, kmax);
                keys_add(r.z, 4 * i + 2, kmin, kmax);
                keys_add(r.w, 4 * i + 3, kmin, kmax);
            }
        };
        size_t i = tid;
        for (; i + stride < nv; i += 2 * stride) {  // both steps' loads in flight
            const float4 p0 = a4[2 * i], q0 = a4[2 * i + 1];
            const float4 p1 = a4[2 * (i + stride)], q1 = a4[2 * (i + stride) + 1];
            step(i, p0, q0);
            step(i + stride, p1, q1);
        }
        if (i < nv) step(i, a4[2 * i], a4[2 * i + 1]);
        done = nv * 4;
    }
    for (size_t i = done + tid; i < n; i += stride) {
        const float v = mag_op<LOG>(a[i], offset);
        d[i] = v;
        if constexpr (KEYS) keys_add(v, i, kmin, kmax);
    }
    if constexpr (KEYS) block_minmax_commit(kmin, kmax, red, keys);
}

// Each thread visits its indices in increasing order, so a running strict
// compare keeps its first occurrence; keys are formed once per thread for the
// block reduction.  Starting from the literal excludes what the reference
// excludes (NaN and values at or beyond it never compare).
struct MinMaxRun {
    float vmin = kMinMaxLiteral, vmax = -kMinMaxLiteral;
    unsigned imin = 0, imax = 0;
    __device__ __forceinline__ void add(float v, unsigned i) {
        if (v < vmin) {
            vmin = v;
            imin = i;
        }
        if (v > vmax) {
            vmax = v;
            imax = i;
        }
    }
    __device__ __forceinline__ void commit(unsigned long long *red, unsigned long long *keys) const {
        block_minmax_commit(min_key(vmin, imin), max_key(vmax, imax), red, keys);
    }
};

// The key reset in front of minmax_kernel: launched in stream order (so no
// earlier reader of the keys can still be running), it lets the min / max
// pass, launched as its programmatic dependent, start streaming at once.
__global__ void minmax_reset_kernel(unsigned long long *keys) {
    keys[0] = 0ull;
    keys[1] = 0ull;
    asm volatile("griddepcontrol.launch_dependents;" ::: "memory");
}

// The input was complete before the reset kernel started (stream order);
// only the keys come from it, so the pass waits for its predecessor grid
// (griddepcontrol.wait, a no-op without programmatic launch) just before it
// commits them.
__global__ void __launch_bounds__(kThreads) minmax_kernel(const float *__restrict__ x, size_t n,
                                                          unsigned long long *keys) {
    __shared__ unsigned long long red[2 * (kThreads / 32)];
    MinMaxRun run;
    const size_t tid = blockIdx.x * (size_t)blockDim.x + threadIdx.x;
    const size_t stride = (size_t)gridDim.x * blockDim.x;
    size_t done = 0;
    if (al16(x)) {
        const size_t nv = n / 4;
        const float4 *x4 = reinterpret_cast<const float4 *>(x);
        // eight independent 16-byte loads in flight before the compares (a
        // read-only stream needs more bytes in flight per thread than a copy;
        // the visiting order per thread stays increasing).  The last batch is
        // predicated, its missing slots NaN, which never compares, so the
        // ragged end costs one round trip rather than one per load.
        constexpr int kBatch = 8;
        const float4 none = make_float4(__int_as_float(0x7fffffff), __int_as_float(0x7fffffff),
                                        __int_as_float(0x7fffffff), __int_as_float(0x7fffffff));
        for (size_t i = tid; i < nv; i += kBatch * stride) {
            float4 v[kBatch];
#pragma unroll
            for (int k = 0; k < kBatch; k++) v[k] = i + k * stride < nv ? x4[i + k * stride] : none;
#pragma unroll
            for (int k = 0; k < kBatch; k++) {
                const unsigned b = (unsigned)(4 * (i + k * stride));
                run.add(v[k].x, b);
                run.add(v[k].y, b + 1);
                run.add(v[k].z, b + 2);
                run.add(v[k].w, b + 3);
            }
        }
        done = nv * 4;
    }
    for (size_t i = done + tid; i < n; i += stride) run.add(x[i], (unsigned)i);
    asm volatile("griddepcontrol.wait;" ::: "memory");  // the keys are reset
    run.commit(red, keys);
}

// dst = (float)(alpha - scl*min) + scl*src, scl = (float)(beta-alpha) / (float)(max-min)
__global__ void __launch_bounds__(kThreads) normalize_kernel(const float *x, float *d, size_t n,
                                                             const unsigned long long *keys,
                                                             double alpha, double beta) {
    pdl_enter();  // the keys come from the grid before
    const double mn = min_key_value(keys[0]), mx = max_key_value(keys[1]);
    const float scl = __fdiv_rn((float)(beta - alpha), (float)(mx - mn));
    const float c = (float)__dsub_rn(alpha, __dmul_rn((double)scl, mn));
    const size_t tid = blockIdx.x * (size_t)blockDim.x + threadIdx.x;
    const size_t stride = (size_t)gridDim.x * blockDim.x;
    size_t done = 0;
    if (al16(x) && al16(d)) {
        const size_t nv = n / 4;
        const float4 *x4 = reinterpret_cast<const float4 *>(x);
        float4 *d4 = reinterpret_cast<float4 *>(d);
        auto step = [&](const float4 v) {
            return make_float4(__fadd_rn(c, __fmul_rn(scl, v.x)), __fadd_rn(c, __fmul_rn(scl, v.y)),
                               __fadd_rn(c, __fmul_rn(scl, v.z)), __fadd_rn(c, __fmul_rn(scl, v.w)));
        };
        // four loads in flight; the last batch predicated (one round trip)
        for (size_t i = tid; i < nv; i += 4 * stride) {
            float4 v[4];
#pragma unroll
            for (int k = 0; k < 4; k++)
                v[k] = i + k * stride < nv ? x4[i + k * stride] : make_float4(0.f, 0.f, 0.f, 0.f);
#pragma unroll
            for (int k = 0; k < 4; k++)
                if (i + k * stride < nv) d4[i + k * stride] = step(v[k]);
        }
        done = nv * 4;
    }
    for (size_t i = done + tid; i < n; i += stride) d[i] = __fadd_rn(c, __fmul_rn(scl, x[i]));
}

bool misaligned(const void *p, size_t a) { return (reinterpret_cast<uintptr_t>(p) % a) != 0; }

// whether [p, p + pb) and [q, q + qb) overlap
bool overlap(const void *p, size_t pb, const void *q, size_t qb) {
    const uintptr_t a = reinterpret_cast<uintptr_t>(p), b = reinterpret_cast<uintptr_t>(q);
    return a < b + qb && b < a + pb;
}

int check_elem(glsfft_context ctx, const void *p0, const void *p1, const void *p2, size_t al,
               int rows, int cols) {
    if (!ctx || !p0 || !p1 || !p2) return GLSFFT_ERROR_INVALID_VALUE;
    if (rows < 1 || cols < 1 || (long long)rows * cols > (1ll << 31)) return GLSFFT_ERROR_SIZE;
    if (misaligned(p0, al) || misaligned(p1, al)) return GLSFFT_ERROR_MISALIGNED;
    return GLSFFT_SUCCESS;
}

// the context's workspace holds the two keys at offset `off`
int keys_at(glsfft_context ctx, size_t off, unsigned long long **keys) {
    const int st = ensure_workspace(ctx, off + 256);
    if (st) return st;
    *keys = reinterpret_cast<unsigned long long *>(static_cast<char *>(ctx->ws) + off);
    return GLSFFT_SUCCESS;
}

}  // namespace

extern "C" {

int glsfft_mul_spectrums(glsfft_context ctx, const void *src0, const void *src1, void *dst,
                         int rows, int cols, int conj, void *stream) {
    int st = check_elem(ctx, src0, src1, dst, sizeof(float2), rows, cols);
    if (!st && misaligned(dst, sizeof(float2))) st = GLSFFT_ERROR_MISALIGNED;
    if (st) return st;
    DeviceGuard g(ctx->device);
    if (!g.ok()) return GLSFFT_ERROR_CUDA;
    const size_t n = (size_t)rows * cols;
    const auto *a = static_cast<const float2 *>(src0);
    const auto *b = static_cast<const float2 *>(src1);
    auto *d = static_cast<float2 *>(dst);
    cudaStream_t s = (cudaStream_t)stream;
    if (conj)
        spec_binary_kernel<1><<<grid_for(spec_binary_kernel<1>, n), kThreads, 0, s>>>(a, b, d, n);
    else
        spec_binary_kernel<0><<<grid_for(spec_binary_kernel<0>, n), kThreads, 0, s>>>(a, b, d, n);
    return cuda_status(cudaGetLastError());
}

int glsfft_mul_spectrums_phase_only(glsfft_context ctx, const void *src0, const void *src1,
                                    void *dst, int rows, int cols, void *stream) {
    int st = check_elem(ctx, src0, src1, dst, sizeof(float2), rows, cols);
    if (!st && misaligned(dst, sizeof(float2))) st = GLSFFT_ERROR_MISALIGNED;
    if (st) return st;
    DeviceGuard g(ctx->device);
    if (!g.ok()) return GLSFFT_ERROR_CUDA;
    const size_t n = (size_t)rows * cols;
    auto kern = spec_binary_kernel<2>;
    kern<<<grid_for(kern, n), kThreads, 0, (cudaStream_t)stream>>>(
        static_cast<const float2 *>(src0), static_cast<const float2 *>(src1),
        static_cast<float2 *>(dst), n);
    return cuda_status(cudaGetLastError());
}

int glsfft_mag_spectrums(glsfft_context ctx, const void *src, float *dst, int rows, int cols,
                         void *stream) {
    int st = check_elem(ctx, src, src, dst, sizeof(float2), rows, cols);
    if (!st && misaligned(dst, sizeof(float))) st = GLSFFT_ERROR_MISALIGNED;
    // the CV_32FC1 output must not overlap the CV_32FC2 input (a new GlsMat, as getDstMat gives)
    if (!st && overlap(src, 8 * (size_t)rows * cols, dst, 4 * (size_t)rows * cols))
        st = GLSFFT_ERROR_INVALID_VALUE;
    if (st) return st;
    DeviceGuard g(ctx->device);
    if (!g.ok()) return GLSFFT_ERROR_CUDA;
    const size_t n = (size_t)rows * cols;
    auto kern = spec_mag_kernel<false, false>;
    kern<<<grid_for(kern, n), kThreads, 0, (cudaStream_t)stream>>>(
        static_cast<const float2 *>(src), dst, n, 0.0f, nullptr);
    return cuda_status(cudaGetLastError());
}

int glsfft_log_mag_spectrums(glsfft_context ctx, const void *src, float *dst, int rows, int cols,
                             float offset, void *stream) {
    int st = check_elem(ctx, src, src, dst, sizeof(float2), rows, cols);
    if (!st && misaligned(dst, sizeof(float))) st = GLSFFT_ERROR_MISALIGNED;
    if (!st && overlap(src, 8 * (size_t)rows * cols, dst, 4 * (size_t)rows * cols))
        st = GLSFFT_ERROR_INVALID_VALUE;
    if (st) return st;
    DeviceGuard g(ctx->device);
    if (!g.ok()) return GLSFFT_ERROR_CUDA;
    const size_t n = (size_t)rows * cols;
    auto kern = spec_mag_kernel<true, false>;
    kern<<<grid_for(kern, n), kThreads, 0, (cudaStream_t)stream>>>(
        static_cast<const float2 *>(src), dst, n, offset, nullptr);
    return cuda_status(cudaGetLastError());
}

int glsfft_min_max_loc_async(glsfft_context ctx, const float *src, int rows, int cols,
                             unsigned long long *d_keys, void *stream) {
    int st = check_elem(ctx, src, src, d_keys, sizeof(float), rows, cols);
    if (!st && misaligned(d_keys, 8)) st = GLSFFT_ERROR_MISALIGNED;
    if (st) return st;
    DeviceGuard g(ctx->device);
    if (!g.ok()) return GLSFFT_ERROR_CUDA;
    const size_t n = (size_t)rows * cols;
    minmax_reset_kernel<<<1, 1, 0, (cudaStream_t)stream>>>(d_keys);
    cudaError_t e = cudaGetLastError();
    if (e != cudaSuccess) return cuda_status(e);
    return cuda_status(launch_maybe_pdl(true, minmax_kernel, grid_for(minmax_kernel, n / 4),
                                        kThreads, 0, (cudaStream_t)stream, src, n, d_keys));
}

int glsfft_min_max_loc(glsfft_context ctx, const float *src, int rows, int cols,
                       double *min_val, double *max_val, int *min_loc, int *max_loc,
                       void *stream) {
    int st = check_elem(ctx, src, src, src, sizeof(float), rows, cols);
    if (st) return st;
    DeviceGuard g(ctx->device);
    if (!g.ok()) return GLSFFT_ERROR_CUDA;
    unsigned long long *keys = nullptr;
    st = keys_at(ctx, 0, &keys);
    if (st) return st;
    st = glsfft_min_max_loc_async(ctx, src, rows, cols, keys, stream);
    if (st) return st;
    unsigned long long *h = reinterpret_cast<unsigned long long *>(ctx->h_result);
    cudaError_t e = cudaMemcpyAsync(h, keys, 2 * sizeof(unsigned long long),
                                    cudaMemcpyDeviceToHost, (cudaStream_t)stream);
    if (e == cudaSuccess) e = cudaStreamSynchronize((cudaStream_t)stream);
    if (e != cudaSuccess) return cuda_status(e);
    const unsigned imin = key_idx(h[0]), imax = key_idx(h[1]);
    if (min_val) *min_val = min_key_value(h[0]);
    if (max_val) *max_val = max_key_value(h[1]);
    if (min_loc) {
        min_loc[0] = (int)(imin % (unsigned)cols);
        min_loc[1] = (int)(imin / (unsigned)cols);
    }
    if (max_loc) {
        max_loc[0] = (int)(imax % (unsigned)cols);
        max_loc[1] = (int)(imax / (unsigned)cols);
    }
    return GLSFFT_SUCCESS;
}

int glsfft_normalize_minmax(glsfft_context ctx, const float *src, float *dst, int rows, int cols,
                            double alpha, double beta, void *stream) {
    int st = check_elem(ctx, src, dst, dst, sizeof(float), rows, cols);
    if (st) return st;
    DeviceGuard g(ctx->device);
    if (!g.ok()) return GLSFFT_ERROR_CUDA;
    unsigned long long *keys = nullptr;
    st = keys_at(ctx, 0, &keys);
    if (!st) st = glsfft_min_max_loc_async(ctx, src, rows, cols, keys, stream);
    if (st) return st;
    const size_t n = (size_t)rows * cols;
    // resident while the min / max pass drains
    return cuda_status(launch_maybe_pdl(true, normalize_kernel, grid_for(normalize_kernel, n),
                                        kThreads, 0, (cudaStream_t)stream, src, dst, n,
                                        (const unsigned long long *)keys, alpha, beta));
}

int glsfft_fft_display(glsfft_context ctx, const float *frame, const float *window, float *dst,
                       int rows, int cols, float offset, void *stream) {
    if (!ctx || !frame || !dst) return GLSFFT_ERROR_INVALID_VALUE;
    int st = check_dims(rows, cols);
    if (st) return st;
    if (misaligned(frame, 4) || misaligned(dst, 4) || (window && misaligned(window, 4)))
        return GLSFFT_ERROR_MISALIGNED;
    DeviceGuard g(ctx->device);
    if (!g.ok()) return GLSFFT_ERROR_CUDA;
    const size_t n = (size_t)rows * cols;
    const size_t spec_bytes = (n * sizeof(float2) + 255) / 256 * 256;
    unsigned long long *keys = nullptr;
    st = keys_at(ctx, spec_bytes, &keys);
    if (st) return st;
    cudaStream_t s = (cudaStream_t)stream;
    float2 *spec = static_cast<float2 *>(ctx->ws);
    // rows: window * frame promoted to complex, FFT of every row, half swap;
    // the row kernel also zeroes the min / max keys
    PassArgs r{};
    r.in0 = frame;
    r.out0 = spec;
    r.window = window;
    r.rows = rows;
    r.cols = cols;
    r.scale = 1.0f;
    r.flags = PF_SHIFT_COLS;
    r.tw = ctx->d_tw;
    r.key = keys;
    r.pdl = 1;  // the three launches are chained by programmatic dependent launch
    cudaError_t e = launch_rows(cols, window ? LD_R1W : LD_R1, ST_C2, r, 1, s);
    if (e != cudaSuccess) return cuda_status(e);
    if (rows > 1) {
        // columns: FFT of every column, half swap, log(|X| + offset) and its min / max
        PassArgs c{};
        c.in0 = spec;
        c.out0 = dst;
        c.rows = rows;
        c.cols = cols;
        c.scale = 1.0f;
        c.flags = PF_SHIFT_ROWS;
        c.key = keys;
        c.tw = ctx->d_tw;
        c.param = offset;
        c.err = ctx->d_status;
        c.stall_ns = ctx->stall_ns;
        c.pdl = 1;  // the plain column kernel; the streamed pass launches as usual
        // 4096-point columns: the streamed pass (TMA-fed, one block per SM)
        e = rows == 4096 && stream_pass_applies(rows, true, c, 1, ST_LOGMAG_MINMAX)
                ? launch_stream_pass(rows, true, c, 1, s, ST_LOGMAG_MINMAX)
                : launch_cols(rows, LD_C2, ST_LOGMAG_MINMAX, c, 1, s);
    } else {
        auto kern = spec_mag_kernel<true, true>;
        kern<<<grid_for(kern, n), kThreads, 0, s>>>(spec, dst, n, offset, keys);
        e = cudaGetLastError();
    }
    if (e != cudaSuccess) return cuda_status(e);
    // normalize(0, 1, NORM_MINMAX) in place
    return cuda_status(launch_maybe_pdl(true, normalize_kernel, grid_for(normalize_kernel, n),
                                        kThreads, 0, s, (const float *)dst, dst, n,
                                        (const unsigned long long *)keys, 0.0, 1.0));
}

}  // extern "C"
