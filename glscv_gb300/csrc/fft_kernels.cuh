// fft_kernels.cuh -- row-pass and column-pass kernels of the 2-D FFT and the
// fused phaseCorrelate kernels, as templates over the line length N.
//
// Reference semantics (glsCV, paths inside that project):
//   gls::fft rows-then-columns Stockham       glsCV/glsFft.cpp:494-671
//   INVERSE = conj in (first pass) / conj out (last pass)   :600, :646
//   SCALE = x 1/N of that dimension at its last stage        :601, :647
//   SHIFT = quadrant swap of the output                      :656-664
//   1-channel input promoted to complex, imag = 0            :684-689
//   window multiply before the FFT       glsCV/glsPhaseCorrelate.cpp:178-184
//   phase-only spectrum, no epsilon      glsCV/glsBasicOperation.cpp:195-206
//   real part of the inverse             glsCV/glsPhaseCorrelate.cpp:202-204
//   first-occurrence argmax              glsCV/glsMinMaxLoc.cpp:65-119
//   FP64 weighted centroid, clamped box  glsCV/glsPhaseCorrelate.cpp:60-137
#pragma once
#include "fft_config.h"
#include "fft_device.cuh"
#include "glsfft_internal.h"
#include "pdl.cuh"
#include "spectrum_device.cuh"

namespace glsfft {

// Shared-memory accessor for a row line: one padding slot per 16 complex
// values keeps the stride-R butterfly writes of the first exchange on
// distinct banks.
struct RowSm {
    static constexpr bool kSplit = false;
    static constexpr int KW = 1;
    float2 *base;
    __device__ __forceinline__ float2 *at(int pos) const { return base + pos + (pos >> 4); }
};
// Column tiles keep [position][column] order (like the image) with the same
// per-16 padding over the linearised index.
template <int W>
struct ColSm {
    static constexpr bool kSplit = false;
    static constexpr int KW = W;
    float2 *base;
    int c;
    __device__ __forceinline__ float2 *at(int pos) const {
        const int i = pos * W + c;
        return base + i + (i >> 4);
    }
};

// Split-exchange accessor for a column tile (real and imaginary parts
// exchanged in turn through a float buffer of half the size), two pad floats
// per 32: with 16 values per thread and radix-16 passes on 2048- and
// 4096-point columns of 8 or 4 per tile, the stores and loads of a warp fall
// on distinct banks.
template <int W>
struct ColSmF {
    static constexpr bool kSplit = true;
    static constexpr int KW = W;
    float *base;
    int c;
    template <int X>
    __device__ __forceinline__ float *at(int pos) const {
        const int i = pos * W + c;
        return base + i + 2 * (i >> 5);
    }
};
__host__ __device__ constexpr int col_split_floats(int count) { return count + 2 * (count >> 5); }

// Whole-line conjugation and scaling behind uniform branches, so the common
// flag-free case spends no instructions per element.
template <int E>
__device__ __forceinline__ void conj_line(float2 (&x)[E], bool on) {
    if (on) {
#pragma unroll
        for (int m = 0; m < E; m++) x[m].y = -x[m].y;
    }
}
template <int E>
__device__ __forceinline__ void finish_line(float2 (&x)[E], float scale, bool conj_out) {
    if (scale != 1.0f) {
        const float si = conj_out ? -scale : scale;
#pragma unroll
        for (int m = 0; m < E; m++) x[m] = make_float2(x[m].x * scale, x[m].y * si);
    } else {
        conj_line(x, conj_out);
    }
}

// Store a line held as x[m] = position t + m*T, optionally half-swapped
// (fftshift along the line): dst + pos*STRIDE for each position pos.
template <int N, int E, int T>
__device__ __forceinline__ void store_line(float2 *dst, size_t stride, const float2 (&x)[E],
                                           int t, bool shift) {
    if (shift) {
#pragma unroll
        for (int m = 0; m < E; m++) dst[(size_t)((t + m * T + (N >> 1)) & (N - 1)) * stride] = x[m];
    } else {
        float2 *p = dst + (size_t)t * stride;
#pragma unroll
        for (int m = 0; m < E; m++) p[(size_t)m * T * stride] = x[m];
    }
}

// Image z of a launch: in1/out1 when set (the two-image phaseCorrelate
// launch), else image z of a contiguous batch starting at in0/out0.
__device__ __forceinline__ const void *image_in(const PassArgs &a, unsigned z) {
    if (z == 1 && a.in1) return a.in1;
    return static_cast<const char *>(a.in0) + (size_t)z * a.in_img_bytes;
}
__device__ __forceinline__ void *image_out(const PassArgs &a, unsigned z) {
    if (z == 1 && a.out1) return a.out1;
    return static_cast<char *>(a.out0) + (size_t)z * a.out_img_bytes;
}

// Launch one pass kernel, with programmatic dependent launch when a.pdl is
// set (the kernel must begin with pdl_enter()).
template <typename Kern>
inline cudaError_t launch_pass(Kern kern, dim3 grid, unsigned threads, size_t smem,
                               cudaStream_t s, const PassArgs &a) {
    return launch_maybe_pdl(a.pdl != 0, kern, grid, dim3(threads), smem, s, a);
}

// ------------------------------------------------------------ load / store
template <int LD>
__device__ __forceinline__ float2 load_elem(const void *img, const float *win, size_t idx) {
    if constexpr (LD == LD_C2) {
        return __ldg(reinterpret_cast<const float2 *>(img) + idx);
    } else if constexpr (LD == LD_R1) {
        return make_float2(__ldg(reinterpret_cast<const float *>(img) + idx), 0.0f);
    } else {  // LD_R1W: window * image, glsBasicOperation.cpp:169
        return make_float2(__ldg(win + idx) * __ldg(reinterpret_cast<const float *>(img) + idx),
                           0.0f);
    }
}

// ---------------------------------------------------- centroid finish
// Decode the argmax key, FP64 weighted centroid over the clamped box in
// row-major order (glsPhaseCorrelate.cpp:60-137), response divided by
// rows*cols (:224-225), shift = center - centroid (:228-230).
// res[0..2] = dx, dy, response; res[3] = peak index as a double, res[4] = peak value.
struct PocBox {
    int px, py, minr, maxr, minc, maxc;
    double peak;
};
__device__ __forceinline__ PocBox poc_box(unsigned long long k, int rows, int cols, int box) {
    PocBox b{0, 0, 0, 0, 0, 0, -3.402823466e+38};
    if (k != 0ull) {
        const unsigned idx = key_index(k);
        b.px = (int)(idx % (unsigned)cols);
        b.py = (int)(idx / (unsigned)cols);
        b.peak = (double)key_value(k);
    }
    b.minr = b.py - (box >> 1);
    b.maxr = b.py + (box >> 1);
    b.minc = b.px - (box >> 1);
    b.maxc = b.px + (box >> 1);
    if (b.minr < 0) b.minr = 0;
    if (b.minc < 0) b.minc = 0;
    if (b.maxr > rows - 1) b.maxr = rows - 1;
    if (b.maxc > cols - 1) b.maxc = cols - 1;
    return b;
}
// One of the centroid's three FP64 sums over the box in the reference's
// row-major order: which = 0: sum of x*v, 1: sum of y*v, 2: sum of v.  The
// products and sums are rounded separately (no fused multiply-add), as the
// reference's CPU code computes them.  The box values come from `vals`
// (row-major, width maxc - minc + 1) when given, else straight from the
// surface through L2 (.cg: the surface was written by other blocks of this
// launch).
__device__ __forceinline__ double poc_sum(const float *surface, int cols, const PocBox &b,
                                          const float *vals, int which) {
    double acc = 0.0;
    const int w = b.maxc - b.minc + 1;
    for (int y = b.minr; y <= b.maxr; y++)
        for (int x = b.minc; x <= b.maxc; x++) {
            const double v = vals ? (double)vals[(y - b.minr) * w + (x - b.minc)]
                                  : (double)__ldcg(surface + (size_t)y * cols + x);
            acc = which == 2 ? __dadd_rn(acc, v)
                             : __dadd_rn(acc, __dmul_rn((double)(which == 0 ? x : y), v));
        }
    return acc;
}

// The three sums at once on one warp, exactly, when no rounding can occur:
// every term x*v, y*v, v of a finite float v and an integer coordinate below
// 2^13 is m * 2^e with an integer m of at most 37 bits; if, for each sum, the
// largest term's leading bit and the smallest term's lowest bit are at most
// 46 binades apart, every partial sum of up to 32 terms is a multiple of the
// lowest bit below 2^53 of it, so the reference's sequential FP64 sum never
// rounds and equals the exact integer sum -- which one warp forms in any
// order (64-bit integers, shuffles) and converts once.  Returns false (on
// every lane) when the box has more than 32 values, a non-finite value, or a
// wider range; the caller then runs the sequential FP64 sums.  GB300's FP64
// pipe makes the sequential chain of 25 dependent additions cost microseconds.
__device__ __forceinline__ bool poc_sums_exact(const float *vals, const PocBox &b, double *out3) {
    const int lane = threadIdx.x & 31;
    const int w = b.maxc - b.minc + 1, n = w * (b.maxr - b.minr + 1);
    if (n > 32) return false;
    unsigned long long mv = 0;  // significand of v
    int e = 0;                  // v = +-mv * 2^e
    bool neg = false, ok = true;
    unsigned cx = 0, cy = 0;
    if (lane < n) {
        const unsigned bits = __float_as_uint(vals[lane]);
        const int e8 = (int)((bits >> 23) & 0xFF);
        ok = e8 != 0xFF;
        neg = bits >> 31;
        mv = (bits & 0x7FFFFFu) | (e8 ? 0x800000u : 0u);
        e = e8 ? e8 - 150 : -149;
        cx = (unsigned)(b.minc + lane % w);
        cy = (unsigned)(b.minr + lane / w);
    }
    if (!__all_sync(0xffffffffu, ok)) return false;
    // the three sums' terms, their top and lowest bits, and the warp-wide
    // extremes: the six reductions run side by side
    unsigned long long m[3];
    int top[3], low[3];
#pragma unroll
    for (int which = 0; which < 3; which++) {
        m[which] = mv * (which == 0 ? cx : which == 1 ? cy : 1u);
        top[which] = m[which] ? e + (63 - __clzll((long long)m[which])) : -100000;
        low[which] = m[which] ? e : 100000;
    }
#pragma unroll
    for (int off = 16; off > 0; off >>= 1) {
#pragma unroll
        for (int which = 0; which < 3; which++) {
            top[which] = max(top[which], __shfl_xor_sync(0xffffffffu, top[which], off));
            low[which] = min(low[which], __shfl_xor_sync(0xffffffffu, low[which], off));
        }
    }
    bool fits = true;
#pragma unroll
    for (int which = 0; which < 3; which++)
        fits = fits && (low[which] == 100000 || top[which] - low[which] <= 46);
    if (!fits) return false;
    // exact integer sums (every term zero: the sum is +0)
    long long q[3];
#pragma unroll
    for (int which = 0; which < 3; which++) {
        const long long t =
            (low[which] != 100000 && m[which]) ? (long long)(m[which] << (e - low[which])) : 0;
        q[which] = neg ? -t : t;
    }
#pragma unroll
    for (int off = 16; off > 0; off >>= 1) {
#pragma unroll
        for (int which = 0; which < 3; which++) q[which] += __shfl_xor_sync(0xffffffffu, q[which], off);
    }
    if (lane == 0) {
#pragma unroll
        for (int which = 0; which < 3; which++) {
            // |sum| < 2^53: exact as a double; times the power of two 2^lo, exact
            const int lo = low[which] == 100000 ? 0 : low[which];
            const double p2 = __longlong_as_double((long long)(lo + 1023) << 52);
            out3[which] = q[which] == 0 ? 0.0 : __dmul_rn((double)q[which], p2);
        }
    }
    return true;
}
// The result from the three sums: response = sum / (rows*cols)
// (:224-225), then sum + DBL_EPSILON divides (:128), shift = center -
// centroid (:228-230).
// part < 0: all of it on this thread; part 0 / 1 / 2: only dx / dy / the
// response, peak index and peak value (three threads of different warps run
// the two FP64 divisions side by side).
__device__ __forceinline__ void poc_result(int rows, int cols, const PocBox &b, double sx,
                                           double sy, double sum, double *res, int part = -1) {
    if (part < 0 || part == 2) {
        res[2] = sum / ((double)rows * (double)cols);
        res[3] = (double)(b.py * cols + b.px);
        res[4] = b.peak;
    }
    sum = __dadd_rn(sum, 2.220446049250313e-16);  // DBL_EPSILON, glsPhaseCorrelate.cpp:128
    if (part < 0 || part == 0) res[0] = __dsub_rn((double)cols / 2.0, sx / sum);
    if (part < 0 || part == 1) res[1] = __dsub_rn((double)rows / 2.0, sy / sum);
}
// boxes up to this many values are read into shared memory by the whole
// block at once (independent L2 reads in flight) before thread 0 sums them
constexpr int kPocBoxCap = 1024;

// The argmax commit of a row pass that writes the correlation surface
// (ST_RE_ARGMAX), and, with a.result set, the centroid in the last block to
// finish.  `best`: this thread's best key; `red`: blockDim.x / 32 shared
// words; `surface`: the pass's output (rows x N floats).
template <int N>
__device__ __forceinline__ void poc_commit_finish(unsigned long long best, unsigned long long *red,
                                                  const PassArgs &a, const float *surface) {
    block_argmax_commit(best, red, a.key);
    if (a.result) {
        // the last block to finish (every block's surface writes and
        // key update are released before its count) computes the centroid
        __shared__ int s_last;
        if (threadIdx.x == 0) {
            // one acquire-release add instead of a full fence and a
            // relaxed add: it releases this block's surface writes
            // (ordered before it by the barrier in the key commit)
            // and, in the last block, acquires every other block's
            unsigned long long prev;
            asm volatile("atom.acq_rel.gpu.global.add.u64 %0, [%1], 1;"
                         : "=l"(prev)
                         : "l"(a.key + 1)
                         : "memory");
            s_last = prev == (unsigned long long)gridDim.x * gridDim.y - 1ull;
        }
        __syncthreads();
        if (s_last) {
            // No fence here: every other block's surface stores and
            // key update precede its release add (its barrier, then
            // thread 0's add), thread 0's acquire add above read the
            // final count, and the barrier orders this block's
            // reads after that acquire.
            __shared__ float s_box[kPocBoxCap];
            const float *surf = surface;
            const PocBox b = poc_box(__ldcg(a.key), a.rows, N, a.box);
            const int w = b.maxc - b.minc + 1, n = w * (b.maxr - b.minr + 1);
            const bool staged = n <= kPocBoxCap;
            if (staged)
                for (int i = threadIdx.x; i < n; i += blockDim.x)
                    s_box[i] = __ldcg(surf + (size_t)(b.minr + i / w) * N + b.minc + i % w);
            __syncthreads();
            // the three FP64 sums: exactly on warp 0 when no rounding
            // can occur, else sequentially on lane 0 of three warps
            // (separate SM partitions); then thread 0 forms the result
            // (a result in mapped host memory needs no system fence:
            // the host reads it after synchronising with the kernel)
            __shared__ double s_sum[3];
            __shared__ int s_exact;
            const int warp = threadIdx.x >> 5, warps = (blockDim.x + 31) >> 5;
            if (warp == 0) {
                const bool ex = staged && poc_sums_exact(s_box, b, s_sum);
                if (threadIdx.x == 0) s_exact = ex;
            }
            __syncthreads();
            if (!s_exact && (threadIdx.x & 31) == 0)
                for (int which = warp; which < 3; which += warps)
                    s_sum[which] = poc_sum(surf, N, b, staged ? s_box : nullptr, which);
            __syncthreads();
            if ((threadIdx.x & 31) == 0 && (warps >= 3 ? warp < 3 : warp == 0))
                poc_result(a.rows, N, b, s_sum[0], s_sum[1], s_sum[2], a.result,
                           warps >= 3 ? warp : -1);
            if (a.done_flag) {
                // the three warps' result stores, then (system scope) the flag
                __syncthreads();
                if (threadIdx.x == 0) {
                    __threadfence_system();
                    *reinterpret_cast<volatile unsigned long long *>(a.done_flag) = 1ull;
                }
            }
        }
    }
}

// ------------------------------------------------------------- row pass
// Block: LINES rows x T threads.  blockIdx.y selects the image.  MB bounds
// the radix (fft_device.cuh).
template <int N, int E, int LINES, int LD, int ST, int MB = 4>
__global__ void __launch_bounds__(LINES *LineFft<N, E>::T)
    fft_rows_kernel(PassArgs a) {
    using F = LineFft<N, E, SyncBlock, MB>;
    constexpr int T = F::T;
    extern __shared__ float4 smem_raw[];
    float2 *smem = reinterpret_cast<float2 *>(smem_raw);
    __shared__ unsigned long long red[(LINES * T + 31) / 32];
    pdl_enter();

    const int l = threadIdx.x / T, t = threadIdx.x % T;
    const int row = blockIdx.x * LINES + l;
    const bool active = row < a.rows;
    const void *in = image_in(a, blockIdx.y);
    void *out = image_out(a, blockIdx.y);
    const bool conj_in = a.flags & PF_CONJ_IN;
    // a complex-output row pass given a key pointer zeroes the two keys for
    // the kernel that follows it (the FFT display's column pass reduces its
    // min / max there), saving a separate reset
    if constexpr (ST == ST_C2) {
        if (a.key && blockIdx.x == 0 && blockIdx.y == 0 && threadIdx.x == 0) {
            a.key[0] = 0ull;
            a.key[1] = 0ull;
        }
    }

    float2 x[E];
    bool staged = false;
    if constexpr ((LD == LD_R1 || LD == LD_R1W) && num_passes(N, MB) > 1 && N >= 4 && N <= 512) {
        // Real input on lines of up to 512 points (8 or more rows per
        // block): the block's rows are staged through the exchange buffer
        // (unused until the first exchange) with 16-byte loads, four times
        // fewer memory requests in flight per thread than per-element
        // loads.  Same values, same products: the result is unchanged.
        // Measured on GB300, phaseCorrelate 512^2: 0.0194 -> 0.0181 ms per
        // call; at 1024 and 2048 points it was slower, so those keep the
        // per-element loads.
        const float *img = reinterpret_cast<const float *>(in);
        if ((reinterpret_cast<uintptr_t>(img) & 15) == 0) {
            const int row0 = blockIdx.x * LINES;
            const int nrows = min(LINES, a.rows - row0);
            const float4 *s4 = reinterpret_cast<const float4 *>(img + (size_t)row0 * N);
            for (int i = threadIdx.x; i < nrows * (N / 4); i += LINES * T)
                smem_raw[i] = __ldg(s4 + i);
            __syncthreads();
            const float *sf = reinterpret_cast<const float *>(smem_raw) + l * N;
#pragma unroll
            for (int m = 0; m < E; m++) {
                const int pos = t + m * T;
                float v = active ? sf[pos] : 0.f;
                if constexpr (LD == LD_R1W)
                    v = active ? __ldg(a.window + (size_t)row * N + pos) * v : 0.f;
                x[m] = make_float2(v, 0.f);
            }
            __syncthreads();  // the first exchange overwrites the staged rows
            staged = true;
        }
    }
    if (!staged) {
#pragma unroll
        for (int m = 0; m < E; m++) {
            const int pos = t + m * T;
            x[m] = active ? load_elem<LD>(in, a.window, (size_t)row * N + pos) : make_float2(0.f, 0.f);
        }
    }
    conj_line(x, conj_in);
    F::run(x, t, RowSm{smem + l * padded_count(N)}, a.tw);

    const int orow = (a.flags & PF_SHIFT_ROWS) ? (row + (a.rows >> 1)) & (a.rows - 1) : row;
    finish_line(x, a.scale, a.flags & PF_CONJ_OUT);
    if constexpr (ST == ST_C2) {
        if (active)
            store_line<N, E, T>(reinterpret_cast<float2 *>(out) + (size_t)orow * N, 1, x, t,
                                a.flags & PF_SHIFT_COLS);
    } else {
        unsigned long long best = 0;
#pragma unroll
        for (int m = 0; m < E; m++) {
            const int pos = t + m * T;
            const int ocol = (a.flags & PF_SHIFT_COLS) ? (pos + (N >> 1)) & (N - 1) : pos;
            const size_t o = (size_t)orow * N + ocol;
            if (active) reinterpret_cast<float *>(out)[o] = x[m].x;
            if constexpr (ST == ST_RE_ARGMAX) {
                unsigned long long k = active ? argmax_key(x[m].x, (unsigned)o) : 0ull;
                best = k > best ? k : best;
            }
        }
        if constexpr (ST == ST_RE_ARGMAX)
            poc_commit_finish<N>(best, red, a, reinterpret_cast<const float *>(out));
    }
}

// ---------------------------------------------------------- column pass
// Block: W adjacent columns x T threads, column index fastest.
template <int N, int E, int W, int LD, int ST, int MB = 4>
__global__ void __launch_bounds__(W *LineFft<N, E>::T)
    fft_cols_kernel(PassArgs a) {
    using F = LineFft<N, E, SyncBlock, MB>;
    constexpr int T = F::T;
    extern __shared__ float4 smem_raw[];
    float2 *smem = reinterpret_cast<float2 *>(smem_raw);
    pdl_enter();

    const int c = threadIdx.x % W, t = threadIdx.x / W;
    const int col = blockIdx.x * W + c;
    const int cols = a.cols;
    const bool active = col < cols;
    const void *in = image_in(a, blockIdx.y);
    void *out = image_out(a, blockIdx.y);
    const bool conj_in = a.flags & PF_CONJ_IN;

    float2 x[E];
#pragma unroll
    for (int m = 0; m < E; m++) {
        const int pos = t + m * T;
        x[m] = active ? load_elem<LD>(in, a.window, (size_t)pos * cols + col) : make_float2(0.f, 0.f);
    }
    conj_line(x, conj_in);
    F::run(x, t, ColSm<W>{smem, c}, a.tw);

    const int ocol = (a.flags & PF_SHIFT_COLS) ? (col + (cols >> 1)) & (cols - 1) : col;
    finish_line(x, a.scale, a.flags & PF_CONJ_OUT);
    if constexpr (ST == ST_C2) {
        if (active)
            store_line<N, E, T>(reinterpret_cast<float2 *>(out) + ocol, (size_t)cols, x, t,
                                a.flags & PF_SHIFT_ROWS);
    } else {
        // the FFT display epilogue: log(|magnitude| + offset) as CV_32FC1
        // (glsBasicOperation.cpp:126-128) and the minMaxLoc keys of what is
        // stored, for the normalisation that follows
        static_assert(ST == ST_LOGMAG_MINMAX, "column-pass store variants: complex, log-magnitude");
        __shared__ unsigned long long red[2 * ((W * T + 31) / 32)];
        MinMaxAny run;
        float *fo = reinterpret_cast<float *>(out);
#pragma unroll
        for (int m = 0; m < E; m++) {
            const int pos = t + m * T;
            const int orow = (a.flags & PF_SHIFT_ROWS) ? (pos + (N >> 1)) & (N - 1) : pos;
            const unsigned o = (unsigned)orow * (unsigned)cols + (unsigned)ocol;
            const float v = spec_log_mag(x[m], a.param);
            if (active) {
                fo[o] = v;
                run.add(v, o);
            }
        }
        block_minmax_commit(run.kmin(), run.kmax(), red, a.key);
    }
}

// conj(P) for the phaseCorrelate column kernels: P = F1 conj(F2) / |F1 conj(F2)|
// (glsBasicOperation.cpp:195-206, every product and sum rounded separately,
// as the shader formula restated in spectrum_device.cuh), conjugated because
// the inverse is taken as conj(FFT(conj P)); |t| = 0 gives 0, not 0/0.
__device__ __forceinline__ float2 poc_conj_phase(float2 f1, float2 f2) {
    const float2 t = spec_mul<true>(f1, f2);
    const float mag = sqrtf(__fadd_rn(__fmul_rn(t.x, t.x), __fmul_rn(t.y, t.y)));
    return mag > 0.f ? make_float2(__fdiv_rn(t.x, mag), -__fdiv_rn(t.y, mag))
                     : make_float2(0.f, 0.f);
}

// --------------------------------------------- fused phaseCorrelate columns
// in0 = row-pass output of src1 (or, with PF_F1_SPECTRUM, its resident full
// 2-D spectrum), in1 = row-pass output of src2.  Each block finishes the
// forward column FFTs of both, forms the phase-only cross spectrum
// P = F1 conj(F2) / |F1 conj(F2)| (glsBasicOperation.cpp:195-206) and runs
// the column FFT of conj(P) -- the first half of the unscaled inverse
// conj(FFT2(conj P)); the row pass that follows only needs the real part,
// which the outer conj leaves unchanged.  Writes to out0 (may alias in0).
// |t| = 0 gives P = 0 (the reference divides 0/0 into NaN).
template <int N, int E, int W>
__global__ void __launch_bounds__(W *LineFft<N, E>::T)
    poc_cols_kernel(PassArgs a) {
    using F = LineFft<N, E>;
    constexpr int T = F::T;
    extern __shared__ float4 smem_raw[];
    float2 *smem = reinterpret_cast<float2 *>(smem_raw);

    const int c = threadIdx.x % W, t = threadIdx.x / W;
    const int col = blockIdx.x * W + c;
    const int cols = a.cols;
    const bool active = col < cols;
    const float2 *f1 = reinterpret_cast<const float2 *>(a.in0);
    const float2 *f2 = reinterpret_cast<const float2 *>(a.in1);
    ColSm<W> sm{smem, c};
    pdl_enter();
    // the argmax key and the block counter of the inverse row pass that follows
    if (a.key && blockIdx.x == 0 && threadIdx.x == 0) {
        a.key[0] = 0ull;
        a.key[1] = 0ull;
    }

    // both lines' loads are issued up front, so the second line's latency
    // overlaps the first line's transform
    float2 x[E], y[E];
#pragma unroll
    for (int m = 0; m < E; m++) {
        const size_t i = (size_t)(t + m * T) * cols + col;
        y[m] = active ? __ldg(f2 + i) : make_float2(0.f, 0.f);
        x[m] = active ? __ldg(f1 + i) : make_float2(0.f, 0.f);
    }
    F::run(y, t, sm, a.tw);
    __syncthreads();  // the exchange buffer is reused by the next line FFT
    if (!(a.flags & PF_F1_SPECTRUM)) {
        F::run(x, t, sm, a.tw);
        __syncthreads();
    }
#pragma unroll
    for (int m = 0; m < E; m++) x[m] = poc_conj_phase(x[m], y[m]);
    F::run(x, t, sm, a.tw);
    float2 *out = reinterpret_cast<float2 *>(a.out0);
#pragma unroll
    for (int m = 0; m < E; m++) {
        const size_t o = (size_t)(t + m * T) * cols + col;
        if (active) out[o] = x[m];
    }
}


}  // namespace glsfft
