// fft_exact.cu -- gls::fft and gls::phaseCorrelate with the reference's own
// line arithmetic ("reference arithmetic" mode).
//
// The default path computes the same transform with its own radix schedule,
// so its results agree with the reference within FP32 rounding.  This mode
// runs, on the GPU, the exact FP32 operations of the reference's CPU
// Stockham routines on every line, so its output is bit-identical to them:
//   * algo 0: the radix-2 DIT type1 Stockham (UnitTest_glsCV/fft_stockhum.cpp:
//     436-538; stage body :477-497), the routine the reference's tests and
//     this repository's oracle are pinned to;
//   * algo 1: the radix-4 DIT Stockham driven one line at a time (:866-1031),
//     the GLSL shader's algorithm (glsCV/glsFft.cpp:203-343): a radix-2
//     pre-pass when log2 N is odd, then radix-4 passes with w^2, w^3 derived
//     in FP32.
// Twiddles are the reference's: w[n] = (cosf, sinf)((float)(-2*pi*n/N)),
// made on the host with its libm (fft_stockhum.cpp:450-455).  Every product
// and sum is rounded separately (no fused multiply-add), as the reference's
// CPU build computes them.  Flags follow gls::fft: INVERSE conjugates the
// input and the output, SCALE multiplies by 1/rows and 1/cols (powers of
// two, exact), SHIFT swaps quadrants.
//
// One block transforms one line in shared memory (two ping-pong buffers,
// 2 x 8 x N bytes), stage by stage with a block barrier between stages; rows
// go from the source into a workspace image, columns from the workspace into
// the destination (so an in-place call with SHIFT cannot race).  It is a
// verification mode, several times slower than the default path.
#include <cuda_runtime.h>

#include <cmath>
#include <vector>

#include "capi_internal.h"
#include "fft_kernels.cuh"
#include "glsfft.h"
#include "glsfft_internal.h"

using namespace glsfft;

namespace {

constexpr int kExactThreads = 256;

__device__ __forceinline__ unsigned insert_zero_bits(unsigned src, int idx, int num) {
    unsigned r = src << num;
    r &= ~((1u << (idx + num)) - 1u);
    r |= src & ((1u << idx) - 1u);
    return r;
}
// separately rounded complex helpers
__device__ __forceinline__ float mul(float a, float b) { return __fmul_rn(a, b); }
__device__ __forceinline__ float add(float a, float b) { return __fadd_rn(a, b); }
__device__ __forceinline__ float sub(float a, float b) { return __fsub_rn(a, b); }

struct ExactArgs {
    const float2 *in;
    float2 *out;
    const float2 *tw;  // n/2 entries, the reference's table for line length n
    int n;             // line length (power of two)
    int lines;         // lines per image
    long long line_step, elem_step;     // input: start of line l = l*line_step, element k at k*elem_step
    long long out_line_step, out_elem_step;
    long long img_elems;                // elements per image (batch stride)
    int conj_in;
    int last;          // apply conj out / scale / shift on store
    float s, sim;      // scale of the real and imaginary parts (last pass)
    int shift_lines, shift_elems;       // output index offsets (halves) on the last pass
};

// radix-2 type1 stage q: y[n] and y[n + N/2] from x[insertZeroBits(n,q,1)]
// and that + 2^q with twiddle w[(n >> q) << q] (fft_stockhum.cpp:477-497)
__device__ __forceinline__ void r2_stage(const float2 *x, float2 *y, int N, int q,
                                         const float2 *w) {
    for (int m = threadIdx.x; m < N / 2; m += blockDim.x) {
        const int iw = (m >> q) << q;
        const int ix0 = (int)insert_zero_bits((unsigned)m, q, 1);
        const int ix1 = ix0 + (1 << q);
        const float2 a = x[ix0], b = x[ix1], t = w[iw];
        const float tr = sub(mul(b.x, t.x), mul(b.y, t.y));
        const float ti = add(mul(b.x, t.y), mul(b.y, t.x));
        y[m] = make_float2(add(a.x, tr), add(a.y, ti));
        y[m + N / 2] = make_float2(sub(a.x, tr), sub(a.y, ti));
    }
}

// radix-4 DIT stage (fft_stockhum.cpp:921-975)
__device__ __forceinline__ void r4_stage(const float2 *x, float2 *y, int N, int q,
                                         const float2 *w) {
    const int M = N / 4;
    for (int m = threadIdx.x; m < M; m += blockDim.x) {
        const int iw = (m >> q) << q;
        const int ix = (int)insert_zero_bits((unsigned)m, q, 2);
        const float2 p0 = x[ix], p1 = x[ix + (1 << q)], p2 = x[ix + 2 * (1 << q)],
                     p3 = x[ix + 3 * (1 << q)];
        const float w1r = w[iw].x, w1i = w[iw].y;
        const float w2r = sub(mul(w1r, w1r), mul(w1i, w1i)), w2i = add(mul(w1r, w1i), mul(w1i, w1r));
        const float w3r = sub(mul(w1r, w2r), mul(w1i, w2i)), w3i = add(mul(w1r, w2i), mul(w1i, w2r));
        const float ar = p0.x, ai = p0.y;
        const float br = sub(mul(p1.x, w1r), mul(p1.y, w1i)), bi = add(mul(p1.x, w1i), mul(p1.y, w1r));
        const float cr = sub(mul(p2.x, w2r), mul(p2.y, w2i)), ci = add(mul(p2.x, w2i), mul(p2.y, w2r));
        const float dr = sub(mul(p3.x, w3r), mul(p3.y, w3i)), di = add(mul(p3.x, w3i), mul(p3.y, w3r));
        const float apcr = add(ar, cr), apci = add(ai, ci), amcr = sub(ar, cr), amci = sub(ai, ci);
        const float bpdr = add(br, dr), bpdi = add(bi, di);
        const float bmdr = sub(br, dr), bmdi = sub(bi, di);
        // j*(b-d) as the reference multiplies it: (0, 1) * (bmdr, bmdi)
        const float jr = sub(mul(0.0f, bmdr), mul(1.0f, bmdi)), ji = add(mul(0.0f, bmdi), mul(1.0f, bmdr));
        y[m] = make_float2(add(apcr, bpdr), add(apci, bpdi));
        y[m + M] = make_float2(sub(amcr, jr), sub(amci, ji));
        y[m + 2 * M] = make_float2(sub(apcr, bpdr), sub(apci, bpdi));
        y[m + 3 * M] = make_float2(add(amcr, jr), add(amci, ji));
    }
}

// the radix-2 pre-pass of an odd log2 N (fft_stockhum.cpp:883-917)
__device__ __forceinline__ void r4_prepass(const float2 *x, float2 *y, int N) {
    const int M = N / 4;
    for (int m = threadIdx.x; m < M; m += blockDim.x) {
        const float2 x0 = x[m], x1 = x[m + M], x2 = x[m + 2 * M], x3 = x[m + 3 * M];
        y[m] = make_float2(add(x0.x, x2.x), add(x0.y, x2.y));
        y[m + M] = make_float2(add(x1.x, x3.x), add(x1.y, x3.y));
        y[m + 2 * M] = make_float2(sub(x0.x, x2.x), sub(x0.y, x2.y));
        y[m + 3 * M] = make_float2(sub(x1.x, x3.x), sub(x1.y, x3.y));
    }
}

template <int ALGO>
__global__ void __launch_bounds__(kExactThreads) exact_lines_kernel(ExactArgs a) {
    extern __shared__ float2 ex_buf[];
    const int N = a.n;
    const int line = blockIdx.x, img = blockIdx.y;
    float2 *A = ex_buf, *B = ex_buf + N;
    const float2 *in = a.in + (size_t)img * a.img_elems + (long long)line * a.line_step;
    for (int k = threadIdx.x; k < N; k += blockDim.x) {
        float2 v = in[(long long)k * a.elem_step];
        if (a.conj_in) v.y = -v.y;
        A[k] = v;
    }
    __syncthreads();
    int Q = 0;
    while ((1 << Q) < N) Q++;
    if (ALGO == 0) {
        for (int q = Q - 1; q >= 0; q--) {
            r2_stage(A, B, N, q, a.tw);
            __syncthreads();
            float2 *t = A;
            A = B;
            B = t;
        }
    } else if (N == 2) {
        if (threadIdx.x == 0) {
            const float2 x0 = A[0], x1 = A[1];
            B[0] = make_float2(add(x0.x, x1.x), add(x0.y, x1.y));
            B[1] = make_float2(sub(x0.x, x1.x), sub(x0.y, x1.y));
        }
        __syncthreads();
        float2 *t = A;
        A = B;
        B = t;
    } else if (N >= 4) {
        if (Q & 1) {
            r4_prepass(A, B, N);
            __syncthreads();
            float2 *t = A;
            A = B;
            B = t;
            Q -= 1;
        }
        for (int q = Q - 2; q >= 0; q -= 2) {
            r4_stage(A, B, N, q, a.tw);
            __syncthreads();
            float2 *t = A;
            A = B;
            B = t;
        }
    }
    float2 *out = a.out + (size_t)img * a.img_elems;
    const int oline = a.last ? (line + a.shift_lines) % a.lines : line;
    for (int k = threadIdx.x; k < N; k += blockDim.x) {
        float2 v = A[k];
        int ok = k;
        if (a.last) {
            v = make_float2(mul(v.x, a.s), mul(v.y, a.sim));
            ok = (k + a.shift_elems) % N;
        }
        out[(long long)oline * a.out_line_step + (long long)ok * a.out_elem_step] = v;
    }
}

cudaError_t launch_exact(int algo, const ExactArgs &a, int images, cudaStream_t s) {
    const size_t smem = 2 * sizeof(float2) * (size_t)a.n;
    const void *k = algo == 0 ? reinterpret_cast<const void *>(exact_lines_kernel<0>)
                              : reinterpret_cast<const void *>(exact_lines_kernel<1>);
    if (smem > 48 * 1024) {
        cudaError_t e = smem_opt_in(k, smem);
        if (e != cudaSuccess) return e;
    }
    const int threads = a.n / 2 < kExactThreads ? (a.n / 2 > 32 ? a.n / 2 : 32) : kExactThreads;
    dim3 grid(a.lines, images);
    if (algo == 0) exact_lines_kernel<0><<<grid, threads, smem, s>>>(a);
    else exact_lines_kernel<1><<<grid, threads, smem, s>>>(a);
    return cudaGetLastError();
}

// The reference's twiddle table for line length n (n/2 entries), made with
// the host libm exactly as fft_stockhum.cpp:450-455 makes it.
std::vector<float2> reference_twiddles(int n) {
    std::vector<float2> w((size_t)(n / 2 > 0 ? n / 2 : 1));
    for (int k = 0; k < n / 2; k++) {
        const float jw = (float)(-2 * M_PI * k / n);
        w[(size_t)k] = make_float2(cosf(jw), sinf(jw));
    }
    return w;
}

// Per-context device copies of the reference tables, one per length.
int exact_tables(glsfft_context ctx, int n, const float2 **out) {
    auto it = ctx->exact_tw.find(n);
    if (it == ctx->exact_tw.end()) {
        const std::vector<float2> w = reference_twiddles(n);
        void *d = nullptr;
        cudaError_t e = cudaMalloc(&d, sizeof(float2) * w.size());
        if (e == cudaSuccess)
            e = cudaMemcpy(d, w.data(), sizeof(float2) * w.size(), cudaMemcpyHostToDevice);
        if (e != cudaSuccess) {
            if (d) cudaFree(d);
            return cuda_status(e);
        }
        it = ctx->exact_tw.emplace(n, static_cast<float2 *>(d)).first;
    }
    *out = it->second;
    return GLSFFT_SUCCESS;
}

}  // namespace

// The exact transform of `count` back-to-back images src -> dst through
// `tmp` (count * rows * cols complex, distinct from src and dst).
int glsfft::fft2d_exact_launch(glsfft_context ctx, const void *src, void *dst, void *tmp,
                               int count, int rows, int cols, int flags, int algo,
                               cudaStream_t s) {
    const bool inv = flags & GLSFFT_INVERSE, scale = flags & GLSFFT_SCALE,
               shift = flags & GLSFFT_SHIFT;
    const bool do_rows = cols > 1, do_cols = rows > 1;
    float sc = 1.0f;
    if (scale) sc = (1.0f / (float)rows) * (1.0f / (float)cols);
    const float sim = inv ? -sc : sc;
    const long long img = (long long)rows * cols;
    const float2 *cur = static_cast<const float2 *>(src);
    if (do_rows) {
        const float2 *tw = nullptr;
        int st = exact_tables(ctx, cols, &tw);
        if (st) return st;
        ExactArgs a{};
        a.in = cur;
        a.out = do_cols ? static_cast<float2 *>(tmp) : static_cast<float2 *>(dst);
        a.tw = tw;
        a.n = cols;
        a.lines = rows;
        a.line_step = cols;
        a.elem_step = 1;
        a.out_line_step = cols;
        a.out_elem_step = 1;
        a.img_elems = img;
        a.conj_in = inv;
        a.last = !do_cols;
        a.s = sc;
        a.sim = sim;
        a.shift_lines = shift ? rows / 2 : 0;
        a.shift_elems = shift ? cols / 2 : 0;
        cudaError_t e = launch_exact(algo, a, count, s);
        if (e != cudaSuccess) return cuda_status(e);
        cur = a.out;
    }
    if (do_cols) {
        const float2 *tw = nullptr;
        int st = exact_tables(ctx, rows, &tw);
        if (st) return st;
        ExactArgs a{};
        a.in = cur;
        a.out = static_cast<float2 *>(dst);
        a.tw = tw;
        a.n = rows;
        a.lines = cols;
        a.line_step = 1;
        a.elem_step = cols;
        a.out_line_step = 1;
        a.out_elem_step = cols;
        a.img_elems = img;
        a.conj_in = inv && !do_rows;
        a.last = 1;
        a.s = sc;
        a.sim = sim;
        a.shift_lines = shift ? cols / 2 : 0;   // lines are columns here
        a.shift_elems = shift ? rows / 2 : 0;
        cudaError_t e = launch_exact(algo, a, count, s);
        if (e != cudaSuccess) return cuda_status(e);
    }
    if (!do_rows && !do_cols) {
        // a 1 x 1 image: the transform is the identity; flags still apply
        ExactArgs a{};
        a.in = cur;
        a.out = static_cast<float2 *>(dst);
        a.n = 1;
        a.lines = 1;
        a.line_step = 1;
        a.elem_step = 1;
        a.out_line_step = 1;
        a.out_elem_step = 1;
        a.img_elems = img;
        a.conj_in = inv;
        a.last = 1;
        a.s = sc;
        a.sim = sim;
        cudaError_t e = launch_exact(0, a, count, s);
        if (e != cudaSuccess) return cuda_status(e);
    }
    return GLSFFT_SUCCESS;
}

// ---------------------------------------------------------- phaseCorrelate
namespace {

// window * frame promoted to complex (glsBasicOperation.cpp:169, glsFft.cpp:
// 684-689), both images; also zeroes the argmax key
__global__ void exact_promote_kernel(const float *a, const float *b, const float *w, float2 *f1,
                                     float2 *f2, size_t n, unsigned long long *key) {
    if (blockIdx.x == 0 && threadIdx.x == 0) key[0] = 0ull;
    for (size_t i = blockIdx.x * (size_t)blockDim.x + threadIdx.x; i < n;
         i += (size_t)gridDim.x * blockDim.x) {
        f1[i] = make_float2(w ? __fmul_rn(w[i], a[i]) : a[i], 0.0f);
        f2[i] = make_float2(w ? __fmul_rn(w[i], b[i]) : b[i], 0.0f);
    }
}

// the phase-only spectrum, no epsilon (glsBasicOperation.cpp:195-206); with
// `guard`, a bin whose |F1 conj F2| is 0 gives 0 instead of 0/0 = NaN
__global__ void exact_poc_kernel(float2 *f1, const float2 *f2, size_t n, int guard) {
    for (size_t i = blockIdx.x * (size_t)blockDim.x + threadIdx.x; i < n;
         i += (size_t)gridDim.x * blockDim.x) {
        const float2 p = spec_poc(f1[i], f2[i]);
        const float2 t = spec_mul<true>(f1[i], f2[i]);
        const bool zero = guard && !(sqrtf(__fadd_rn(__fmul_rn(t.x, t.x), __fmul_rn(t.y, t.y))) > 0.f);
        f1[i] = zero ? make_float2(0.f, 0.f) : p;
    }
}

// the real part (glsPhaseCorrelate.cpp:202-204) and its first-max key
__global__ void __launch_bounds__(kExactThreads) exact_real_argmax_kernel(const float2 *c,
                                                                         float *surface, size_t n,
                                                                         unsigned long long *key) {
    __shared__ unsigned long long red[kExactThreads / 32];
    unsigned long long best = 0ull;
    for (size_t i = blockIdx.x * (size_t)blockDim.x + threadIdx.x; i < n;
         i += (size_t)gridDim.x * blockDim.x) {
        const float v = c[i].x;
        surface[i] = v;
        const unsigned long long k = argmax_key(v, (unsigned)i);
        best = k > best ? k : best;
    }
    block_argmax_commit(best, red, key);
}

// the centroid from the key and the surface: one block
__global__ void __launch_bounds__(kExactThreads) exact_centroid_kernel(const float *surface,
                                                                      int rows, int cols, int box,
                                                                      const unsigned long long *key,
                                                                      double *result) {
    __shared__ float s_box[kPocBoxCap];
    __shared__ double s_sum[3];
    const PocBox b = poc_box(key[0], rows, cols, box);
    const int w = b.maxc - b.minc + 1, n = w * (b.maxr - b.minr + 1);
    const bool staged = n <= kPocBoxCap;
    if (staged)
        for (int i = threadIdx.x; i < n; i += blockDim.x)
            s_box[i] = surface[(size_t)(b.minr + i / w) * cols + b.minc + i % w];
    __syncthreads();
    const int warp = threadIdx.x >> 5, warps = (blockDim.x + 31) >> 5;
    if ((threadIdx.x & 31) == 0)
        for (int which = warp; which < 3; which += warps)
            s_sum[which] = poc_sum(surface, cols, b, staged ? s_box : nullptr, which);
    __syncthreads();
    if (threadIdx.x == 0) poc_result(rows, cols, b, s_sum[0], s_sum[1], s_sum[2], result);
}

int elem_grid(size_t n) {
    const size_t b = (n + kExactThreads - 1) / kExactThreads;
    return (int)(b < 4096 ? (b ? b : 1) : 4096);
}

}  // namespace

extern "C" {

int glsfft_fft2d_reference(glsfft_context ctx, const void *src, void *dst, int count, int rows,
                           int cols, int flags, int algo, void *stream) {
    int st = check_fft_args(src, dst, rows, cols, flags, false);
    if (st) return st;
    if (!ctx || count < 1 || count > kMaxBatch || (algo != 0 && algo != 1))
        return GLSFFT_ERROR_INVALID_VALUE;
    DeviceGuard g(ctx->device);
    if (!g.ok()) return GLSFFT_ERROR_CUDA;
    const size_t bytes = (size_t)count * rows * cols * sizeof(float2);
    st = ensure_workspace(ctx, bytes);
    if (st) return st;
    return fft2d_exact_launch(ctx, src, dst, ctx->ws, count, rows, cols, flags, algo,
                              (cudaStream_t)stream);
}

int glsfft_phase_correlate_reference(glsfft_context ctx, const float *src1, const float *src2,
                                     const float *window, int rows, int cols, int box, int algo,
                                     double *dx, double *dy, double *response, void *stream) {
    const int guard = (algo & GLSFFT_REFERENCE_ZERO_GUARD) ? 1 : 0;
    algo &= ~GLSFFT_REFERENCE_ZERO_GUARD;
    if (!dx || !dy || (algo != 0 && algo != 1)) return GLSFFT_ERROR_INVALID_VALUE;
    int st = check_poc_args(ctx, src1, src2, window, rows, cols, box);
    if (st) return st;
    DeviceGuard g(ctx->device);
    if (!g.ok()) return GLSFFT_ERROR_CUDA;
    const size_t n = (size_t)rows * cols;
    const size_t cplx = (n * sizeof(float2) + 255) / 256 * 256;
    const size_t surf = (n * sizeof(float) + 255) / 256 * 256;
    st = ensure_workspace(ctx, 3 * cplx + surf + 256);
    if (st) return st;
    char *ws = static_cast<char *>(ctx->ws);
    float2 *f1 = reinterpret_cast<float2 *>(ws);
    float2 *f2 = reinterpret_cast<float2 *>(ws + cplx);
    float2 *tmp = reinterpret_cast<float2 *>(ws + 2 * cplx);
    float *surface = reinterpret_cast<float *>(ws + 3 * cplx);
    auto *key = reinterpret_cast<unsigned long long *>(ws + 3 * cplx + surf);
    cudaStream_t s = (cudaStream_t)stream;
    exact_promote_kernel<<<elem_grid(n), kExactThreads, 0, s>>>(src1, src2, window, f1, f2, n, key);
    cudaError_t e = cudaGetLastError();
    if (e != cudaSuccess) return cuda_status(e);
    st = fft2d_exact_launch(ctx, f1, f1, tmp, 1, rows, cols, 0, algo, s);
    if (!st) st = fft2d_exact_launch(ctx, f2, f2, tmp, 1, rows, cols, 0, algo, s);
    if (st) return st;
    exact_poc_kernel<<<elem_grid(n), kExactThreads, 0, s>>>(f1, f2, n, guard);
    e = cudaGetLastError();
    if (e != cudaSuccess) return cuda_status(e);
    // fft(C, C, INVERSE | SHIFT), unscaled (glsPhaseCorrelate.cpp:199)
    st = fft2d_exact_launch(ctx, f1, f1, tmp, 1, rows, cols, GLSFFT_INVERSE | GLSFFT_SHIFT, algo, s);
    if (st) return st;
    exact_real_argmax_kernel<<<elem_grid(n), kExactThreads, 0, s>>>(f1, surface, n, key);
    exact_centroid_kernel<<<1, kExactThreads, 0, s>>>(surface, rows, cols, box, key,
                                                      ctx->h_result_dev);
    e = cudaGetLastError();
    if (e == cudaSuccess) e = cudaStreamSynchronize(s);
    if (e != cudaSuccess) return cuda_status(e);
    ctx->surface = surface;
    ctx->surface_count = n;
    *dx = ctx->h_result[0];
    *dy = ctx->h_result[1];
    if (response) *response = ctx->h_result[2];
    return GLSFFT_SUCCESS;
}

}  // extern "C"
