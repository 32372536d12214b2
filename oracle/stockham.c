/*
 * oracle/stockham.c -- CPU restatement of glsCV's FFT / phaseCorrelate path.
 *
 * TEST INFRASTRUCTURE ONLY.  This file is the parity checker for the CUDA
 * path and the timed CPU baseline.  Only tests/, __graft_entry__.smoke() and
 * bench.py's CPU-baseline leg may load it; the product library never does.
 *
 * What is restated, and from where (paths inside the glsCV project):
 *   - r2t1_line / oracle_fft_r2t1_square: the FP32 radix-2 DIT Stockham
 *     "type1" of UnitTest_glsCV/fft_stockhum.cpp:436-538 (twiddles :450-455,
 *     row loop :462-498, column loop :502-533, result buf[0] :536).  The
 *     square entry point performs the same float operations in the same
 *     order as the reference function, so with -ffp-contract=off both give
 *     bit-identical results (pinned by tests/test_oracle.py against the
 *     reference compiled from its own source into oracle/_ref).
 *   - r4_line: the FP32 radix-4 DIT Stockham of fft_stockhum.cpp:771-1033
 *     (the algorithm of the GLSL shader glsCV/glsFft.cpp:203-343), driven
 *     one line at a time, which is how it is correct for every shape.
 *   - oracle_fft2d: gls::fft semantics, glsCV/glsFft.cpp:494-708:
 *     INVERSE = conj(FFT(conj x)) (:600, :646), SCALE = x1/N per dimension
 *     (:601, :647), SHIFT = quadrant swap (:656-664; half swap for 1-D lines,
 *     as the reference test's fftShift does, unittest_glsFft.cpp:44-98).
 *   - oracle_phase_correlate: glsCV/glsPhaseCorrelate.cpp:142-231 with the
 *     POC shader of glsCV/glsBasicOperation.cpp:195-206, the strict '>'
 *     first-occurrence argmax of glsCV/glsMinMaxLoc.cpp:65-119 and the FP64
 *     weightedCentroid of glsPhaseCorrelate.cpp:60-137.
 *
 * Complex data is interleaved float (re, im), row-major, like CV_32FC2.
 * OpenMP parallelises rows/columns exactly where the reference does
 * (fft_stockhum.cpp:462, :502); every line is computed independently, so
 * results do not depend on the thread count.
 */
#include <float.h>
#include <math.h>
#include <stdint.h>
#include <stdlib.h>
#include <string.h>
#ifdef _OPENMP
#include <omp.h>
#endif

#ifndef M_PI
#define M_PI 3.14159265358979323846
#endif

#define ORACLE_SCALE 2   /* DFT_SCALE   */
#define ORACLE_INVERSE 1 /* DFT_INVERSE */
#define ORACLE_SHIFT 64  /* GLS_FFT_SHIFT */

static int is_pow2(int x) { return x > 0 && (x & (x - 1)) == 0; }
static int ilog2(int n) { int q = 0; while ((1 << q) < n) q++; return q; }

/* fft_stockhum.cpp:262-272: insert `num` zero bits at bit position `idx`. */
static unsigned insert_zero_bits(unsigned src, int idx, int num) {
    unsigned ret = src << num;
    ret &= ~((1u << (idx + num)) - 1u);
    ret |= src & ((1u << idx) - 1u);
    return ret;
}

/* fft_stockhum.cpp:450-455: FP32 twiddles from an FP32-rounded angle. */
static void make_twiddles(float *w, int count, int N) {
    for (int n = 0; n < count; n++) {
        float jw = (float)(-2 * M_PI * n / N);
        w[2 * n + 0] = cosf(jw);
        w[2 * n + 1] = sinf(jw);
    }
}

/* One radix-2 butterfly stage body of fft_stockhum.cpp:477-497. */
static void r2t1_stage(const float *x, float *y, int N, int q, long stride,
                       const float *w) {
    for (int n = 0; n < N / 2; n++) {
        int iw = (n >> q) << q;
        long ix0 = (long)insert_zero_bits((unsigned)n, q, 1);
        long ix1 = ix0 + (1 << q);
        long iy0 = n;
        long iy1 = iy0 + N / 2;
        ix0 *= stride; ix1 *= stride; iy0 *= stride; iy1 *= stride;
        float xr = x[2 * ix1], xi = x[2 * ix1 + 1];
        float wr = w[2 * iw], wi = w[2 * iw + 1];
        float tr = xr * wr - xi * wi;
        float ti = xr * wi + xi * wr;
        float ar = x[2 * ix0], ai = x[2 * ix0 + 1];
        y[2 * iy0] = ar + tr;     y[2 * iy0 + 1] = ai + ti;
        y[2 * iy1] = ar - tr;     y[2 * iy1 + 1] = ai - ti;
    }
}

/*
 * Square N x N radix-2 type1 Stockham, fft_stockhum.cpp:436-538.
 * Rows ping-pong from bank 0, columns start at bank Q&1 (:505), so the
 * result always lands in buf[0] (:536).  Forward, unscaled.
 */
int oracle_fft_r2t1_square(const float *src, float *dst, int N) {
    if (!is_pow2(N)) return -1;
    size_t n2 = (size_t)N * N * 2;
    float *buf[2];
    buf[0] = (float *)malloc(n2 * sizeof(float));
    buf[1] = (float *)malloc(n2 * sizeof(float));
    float *w = (float *)malloc(sizeof(float) * 2 * (N / 2 > 0 ? N / 2 : 1));
    if (!buf[0] || !buf[1] || !w) { free(buf[0]); free(buf[1]); free(w); return -2; }
    memcpy(buf[0], src, n2 * sizeof(float));
    make_twiddles(w, N / 2, N);
    int Q = ilog2(N);
#pragma omp parallel for schedule(static)
    for (int row = 0; row < N; row++) {
        int bank = 0;
        for (int q = Q - 1; q >= 0; q--, bank ^= 1)
            r2t1_stage(buf[bank] + (size_t)2 * row * N, buf[bank ^ 1] + (size_t)2 * row * N,
                       N, q, 1, w);
    }
#pragma omp parallel for schedule(static)
    for (int col = 0; col < N; col++) {
        int bank = Q & 1;
        for (int q = Q - 1; q >= 0; q--, bank ^= 1)
            r2t1_stage(buf[bank] + (size_t)2 * col, buf[bank ^ 1] + (size_t)2 * col, N, q, N, w);
    }
    memcpy(dst, buf[0], n2 * sizeof(float));
    free(buf[0]); free(buf[1]); free(w);
    return 0;
}

/*
 * One line of length N (elements `stride` complex apart) through the
 * radix-2 type1 stages.  `x` holds the line and receives the result; `tmp`
 * is a contiguous scratch line of N complex.  Same float operations as the
 * square routine, so a square image done line by line matches it bit for bit.
 */
static void r2t1_line(float *x, long stride, float *tmp, int N, const float *w) {
    int Q = ilog2(N);
    /* gather into tmp (contiguous), ping-pong between tmp and tmp2 */
    float *a = tmp, *b = tmp + 2 * (size_t)N;
    for (int i = 0; i < N; i++) { a[2 * i] = x[2 * i * stride]; a[2 * i + 1] = x[2 * i * stride + 1]; }
    for (int q = Q - 1; q >= 0; q--) { r2t1_stage(a, b, N, q, 1, w); float *t = a; a = b; b = t; }
    for (int i = 0; i < N; i++) { x[2 * i * stride] = a[2 * i]; x[2 * i * stride + 1] = a[2 * i + 1]; }
}

/*
 * One line through the radix-4 DIT Stockham of fft_stockhum.cpp:866-1031:
 * a radix-2 pre-pass when log2 N is odd (:883-917), then radix-4 passes with
 * in-index insertZeroBits(n,q,2)+k*2^q, twiddle w[(n>>q)<<q] and its square
 * and cube, out-index n+k*N/4 (:921-975).  N >= 4 (the reference's tiling
 * floor, glsFft.cpp:494-532); N = 2 is one plain butterfly.
 */
static void r4_line(float *x, long stride, float *tmp, int N, const float *w) {
    float *a = tmp, *b = tmp + 2 * (size_t)N;
    for (int i = 0; i < N; i++) { a[2 * i] = x[2 * i * stride]; a[2 * i + 1] = x[2 * i * stride + 1]; }
    if (N == 2) {
        float r0 = a[0], i0 = a[1], r1 = a[2], i1 = a[3];
        b[0] = r0 + r1; b[1] = i0 + i1; b[2] = r0 - r1; b[3] = i0 - i1;
        float *t = a; a = b; b = t;
    } else if (N >= 4) {
        int Q = ilog2(N);
        int M = N / 4;
        if (Q % 2) {
            for (int n = 0; n < M; n++) {
                const float *x0 = a + 2 * (n + 0 * M), *x1 = a + 2 * (n + 1 * M);
                const float *x2 = a + 2 * (n + 2 * M), *x3 = a + 2 * (n + 3 * M);
                float *y0 = b + 2 * (n + 0 * M), *y1 = b + 2 * (n + 1 * M);
                float *y2 = b + 2 * (n + 2 * M), *y3 = b + 2 * (n + 3 * M);
                float o0r = x0[0] + x2[0], o0i = x0[1] + x2[1];
                float o1r = x1[0] + x3[0], o1i = x1[1] + x3[1];
                float o2r = x0[0] - x2[0], o2i = x0[1] - x2[1];
                float o3r = x1[0] - x3[0], o3i = x1[1] - x3[1];
                y0[0] = o0r; y0[1] = o0i; y1[0] = o1r; y1[1] = o1i;
                y2[0] = o2r; y2[1] = o2i; y3[0] = o3r; y3[1] = o3i;
            }
            float *t = a; a = b; b = t;
            Q -= 1;
        }
        for (int q = Q - 2; q >= 0; q -= 2) {
            for (int n = 0; n < M; n++) {
                int iw = (n >> q) << q;
                int ix = (int)insert_zero_bits((unsigned)n, q, 2);
                const float *p0 = a + 2 * (ix + (1 << q) * 0), *p1 = a + 2 * (ix + (1 << q) * 1);
                const float *p2 = a + 2 * (ix + (1 << q) * 2), *p3 = a + 2 * (ix + (1 << q) * 3);
                float w1r = w[2 * iw], w1i = w[2 * iw + 1];
                float w2r = w1r * w1r - w1i * w1i, w2i = w1r * w1i + w1i * w1r;
                float w3r = w1r * w2r - w1i * w2i, w3i = w1r * w2i + w1i * w2r;
                float ar = p0[0], ai = p0[1];
                float br = p1[0] * w1r - p1[1] * w1i, bi = p1[0] * w1i + p1[1] * w1r;
                float cr = p2[0] * w2r - p2[1] * w2i, ci = p2[0] * w2i + p2[1] * w2r;
                float dr = p3[0] * w3r - p3[1] * w3i, di = p3[0] * w3i + p3[1] * w3r;
                float apcr = ar + cr, apci = ai + ci, amcr = ar - cr, amci = ai - ci;
                float bpdr = br + dr, bpdi = bi + di;
                /* j*(b-d) = (-(bi-di), (br-dr)); mul((0,1), v), fft_stockhum.cpp:571-577 */
                float bmdr = br - dr, bmdi = bi - di;
                float jr = 0.0f * bmdr - 1.0f * bmdi, ji = 0.0f * bmdi + 1.0f * bmdr;
                float *y0 = b + 2 * (n + 0 * M), *y1 = b + 2 * (n + 1 * M);
                float *y2 = b + 2 * (n + 2 * M), *y3 = b + 2 * (n + 3 * M);
                y0[0] = apcr + bpdr; y0[1] = apci + bpdi;
                y1[0] = amcr - jr;   y1[1] = amci - ji;
                y2[0] = apcr - bpdr; y2[1] = apci - bpdi;
                y3[0] = amcr + jr;   y3[1] = amci + ji;
            }
            float *t = a; a = b; b = t;
        }
    }
    for (int i = 0; i < N; i++) { x[2 * i * stride] = a[2 * i]; x[2 * i * stride + 1] = a[2 * i + 1]; }
}

typedef void (*line_fn)(float *, long, float *, int, const float *);

/* Forward, unscaled transform of every row, then every column. */
static int fft2d_lines(float *img, int rows, int cols, line_fn fn) {
    int maxn = rows > cols ? rows : cols;
    float *wr = (float *)malloc(sizeof(float) * 2 * (cols > 1 ? cols : 1));
    float *wc = (float *)malloc(sizeof(float) * 2 * (rows > 1 ? rows : 1));
    if (!wr || !wc) { free(wr); free(wc); return -2; }
    make_twiddles(wr, cols / 2 > 0 ? cols / 2 : 0, cols);
    make_twiddles(wc, rows / 2 > 0 ? rows / 2 : 0, rows);
    int err = 0;
    if (cols > 1) {
#pragma omp parallel
        {
            float *tmp = (float *)malloc(sizeof(float) * 4 * (size_t)maxn);
            if (!tmp) {
#pragma omp atomic write
                err = -2;
            } else {
#pragma omp for schedule(static)
                for (int r = 0; r < rows; r++) fn(img + (size_t)2 * r * cols, 1, tmp, cols, wr);
                free(tmp);
            }
        }
    }
    if (rows > 1 && !err) {
#pragma omp parallel
        {
            float *tmp = (float *)malloc(sizeof(float) * 4 * (size_t)maxn);
            if (!tmp) {
#pragma omp atomic write
                err = -2;
            } else {
#pragma omp for schedule(static)
                for (int c = 0; c < cols; c++) fn(img + (size_t)2 * c, cols, tmp, rows, wc);
                free(tmp);
            }
        }
    }
    free(wr); free(wc);
    return err;
}

/* Quadrant swap (fftshift for even sizes), glsFft.cpp:656-664; a 1-D line
 * swaps its halves like unittest_glsFft.cpp:59-75. */
static void shift2d(float *img, int rows, int cols) {
    int hr = rows >> 1, hc = cols >> 1;
    size_t n = (size_t)rows * cols;
    float *t = (float *)malloc(n * 2 * sizeof(float));
    if (!t) return;
    for (int r = 0; r < rows; r++)
        for (int c = 0; c < cols; c++) {
            int rr = (r + hr) % rows, cc = (c + hc) % cols;
            t[2 * ((size_t)rr * cols + cc)] = img[2 * ((size_t)r * cols + c)];
            t[2 * ((size_t)rr * cols + cc) + 1] = img[2 * ((size_t)r * cols + c) + 1];
        }
    memcpy(img, t, n * 2 * sizeof(float));
    free(t);
}

/*
 * gls::fft(src, dst, flag) on a complex rows x cols image (glsFft.cpp:675-708)
 * with `algo` 0 = radix-2 type1 lines (bit-identical to the reference's
 * square routine), 1 = radix-4 lines (the shader's algorithm).
 * INVERSE conjugates the input and the output, SCALE multiplies by 1/rows
 * and 1/cols (exact powers of two), SHIFT swaps quadrants / halves.
 */
int oracle_fft2d(const float *src, float *dst, int rows, int cols, int flags, int algo) {
    if (!is_pow2(rows) || !is_pow2(cols)) return -1;
    size_t n = (size_t)rows * cols;
    if (dst != src) memcpy(dst, src, n * 2 * sizeof(float));
    if (flags & ORACLE_INVERSE)
        for (size_t i = 0; i < n; i++) dst[2 * i + 1] = -dst[2 * i + 1];
    int err = fft2d_lines(dst, rows, cols, algo == 1 ? r4_line : r2t1_line);
    if (err) return err;
    if (flags & (ORACLE_INVERSE | ORACLE_SCALE)) {
        float s = 1.0f;
        if (flags & ORACLE_SCALE) s = (1.0f / (float)rows) * (1.0f / (float)cols);
        float sim = (flags & ORACLE_INVERSE) ? -s : s;
        for (size_t i = 0; i < n; i++) { dst[2 * i] *= s; dst[2 * i + 1] *= sim; }
    }
    if (flags & ORACLE_SHIFT) shift2d(dst, rows, cols);
    return 0;
}

/*
 * weightedCentroid, glsPhaseCorrelate.cpp:60-137: clamped box around the
 * peak, FP64 sums in row-major order, +DBL_EPSILON before the divide.
 */
static void weighted_centroid(const float *c, int rows, int cols, int px, int py, int box,
                              double *cx, double *cy, double *sum_out) {
    int minr = py - (box >> 1), maxr = py + (box >> 1);
    int minc = px - (box >> 1), maxc = px + (box >> 1);
    if (minr < 0) minr = 0;
    if (minc < 0) minc = 0;
    if (maxr > rows - 1) maxr = rows - 1;
    if (maxc > cols - 1) maxc = cols - 1;
    double sx = 0.0, sy = 0.0, s = 0.0;
    for (int y = minr; y <= maxr; y++)
        for (int x = minc; x <= maxc; x++) {
            double v = (double)c[(size_t)y * cols + x];
            sx += (double)x * v;
            sy += (double)y * v;
            s += v;
        }
    *sum_out = s;
    s += DBL_EPSILON;
    *cx = sx / s;
    *cy = sy / s;
}

/*
 * minMaxLoc max/maxLoc, glsMinMaxLoc.cpp:65-119: per-row scan then a scan
 * over rows, both with strict '>' from -FLT_MAX, so ties resolve to the first
 * row-major index and NaN never wins.
 */
void oracle_max_loc(const float *c, int rows, int cols, int *px, int *py, float *maxval) {
    float best = -FLT_MAX;
    int bx = 0, by = 0;
    for (int y = 0; y < rows; y++) {
        float rmax = -FLT_MAX;
        int rx = 0;
        for (int x = 0; x < cols; x++) {
            float v = c[(size_t)y * cols + x];
            if (v > rmax) { rmax = v; rx = x; }
        }
        if (rmax > best) { best = rmax; bx = rx; by = y; }
    }
    *px = bx; *py = by;
    if (maxval) *maxval = best;
}

/*
 * gls::phaseCorrelate(src1, src2, window, &response),
 * glsPhaseCorrelate.cpp:142-231.  a, b, window: rows x cols float
 * (window may be NULL).  `box` is the centroid box edge (the reference uses
 * 5, :219).  `algo` picks the line FFT as in oracle_fft2d.  zero_guard = 0
 * keeps the reference's phase-only division without epsilon (a bin with
 * |F1 conj F2| = 0 becomes NaN and poisons the whole surface); 1 maps such a
 * bin to 0, the GB300 path's documented behaviour.  Optional outputs: the
 * real correlation surface (rows*cols floats) and the peak.
 */
int oracle_phase_correlate(const float *a, const float *b, const float *window, int rows,
                           int cols, int box, int algo, int zero_guard, double *dx, double *dy,
                           double *response, float *surface, int *peak_xy) {
    if (!is_pow2(rows) || !is_pow2(cols)) return -1;
    size_t n = (size_t)rows * cols;
    float *f1 = (float *)malloc(n * 2 * sizeof(float));
    float *f2 = (float *)malloc(n * 2 * sizeof(float));
    float *re = (float *)malloc(n * sizeof(float));
    if (!f1 || !f2 || !re) { free(f1); free(f2); free(re); return -2; }
    /* window multiply (glsBasicOperation.cpp:169, :265-272) and the
     * 1-channel -> complex promotion with imag = 0 (glsFft.cpp:684-689) */
    for (size_t i = 0; i < n; i++) {
        float wv = window ? window[i] : 1.0f;
        f1[2 * i] = window ? wv * a[i] : a[i]; f1[2 * i + 1] = 0.0f;
        f2[2 * i] = window ? wv * b[i] : b[i]; f2[2 * i + 1] = 0.0f;
    }
    int err = oracle_fft2d(f1, f1, rows, cols, 0, algo);
    if (!err) err = oracle_fft2d(f2, f2, rows, cols, 0, algo);
    if (err) { free(f1); free(f2); free(re); return err; }
    /* mulSpectrumsPhaseOnly, shader op 8, glsBasicOperation.cpp:195-206 */
    for (size_t i = 0; i < n; i++) {
        float s0r = f1[2 * i], s0i = f1[2 * i + 1], s1r = f2[2 * i], s1i = f2[2 * i + 1];
        float tr = s0r * s1r + s0i * s1i;
        float ti = -s0r * s1i + s0i * s1r;
        float mag = sqrtf(tr * tr + ti * ti);
        if (zero_guard && !(mag > 0.0f)) { f1[2 * i] = 0.0f; f1[2 * i + 1] = 0.0f; continue; }
        f1[2 * i] = tr / mag; /* 0/0 -> NaN without the guard, as the shader does */
        f1[2 * i + 1] = ti / mag;
    }
    /* fft(C, C, INVERSE | SHIFT), unscaled (glsPhaseCorrelate.cpp:199) */
    err = oracle_fft2d(f1, f1, rows, cols, ORACLE_INVERSE | ORACLE_SHIFT, algo);
    if (err) { free(f1); free(f2); free(re); return err; }
    for (size_t i = 0; i < n; i++) re[i] = f1[2 * i]; /* split -> real plane */
    int px, py;
    oracle_max_loc(re, rows, cols, &px, &py, NULL);
    double cx, cy, s;
    weighted_centroid(re, rows, cols, px, py, box, &cx, &cy, &s);
    if (response) *response = s / ((double)rows * (double)cols);
    *dx = (double)cols / 2.0 - cx;
    *dy = (double)rows / 2.0 - cy;
    if (surface) memcpy(surface, re, n * sizeof(float));
    if (peak_xy) { peak_xy[0] = px; peak_xy[1] = py; }
    free(f1); free(f2); free(re);
    return 0;
}

/*
 * The tail of gls::phaseCorrelate on a given correlation surface
 * (glsPhaseCorrelate.cpp:205-231): first-max location, clamped-box FP64
 * weighted centroid, response = sum / (rows*cols), shift = center - centroid.
 * Lets a test check the GPU's centroid arithmetic on the GPU's own surface.
 */
void oracle_centroid(const float *surface, int rows, int cols, int box, double *dx, double *dy,
                     double *response, int *peak_xy) {
    int px, py;
    oracle_max_loc(surface, rows, cols, &px, &py, NULL);
    double cx, cy, s;
    weighted_centroid(surface, rows, cols, px, py, box, &cx, &cy, &s);
    *response = s / ((double)rows * (double)cols);
    *dx = (double)cols / 2.0 - cx;
    *dy = (double)rows / 2.0 - cy;
    peak_xy[0] = px;
    peak_xy[1] = py;
}

/* Element-wise helpers for the spectrum-op family
 * (glsBasicOperation.cpp:153-212, :320-351). */
void oracle_mul_spectrums(const float *a, const float *b, float *out, size_t n, int conj) {
    for (size_t i = 0; i < n; i++) {
        float ar = a[2 * i], ai = a[2 * i + 1], br = b[2 * i], bi = b[2 * i + 1];
        if (conj) { out[2 * i] = ar * br + ai * bi; out[2 * i + 1] = -ar * bi + ai * br; }
        else      { out[2 * i] = ar * br - ai * bi; out[2 * i + 1] = ar * bi + ai * br; }
    }
}

/* mulSpectrumsPhaseOnly (glsCV/glsBasicOperation.cpp:195-206, shader op 8):
 * t = a * conj(b), out = t / sqrt(t.re^2 + t.im^2), no epsilon (0/0 = NaN). */
void oracle_mul_spectrums_poc(const float *a, const float *b, float *out, size_t n) {
    for (size_t i = 0; i < n; i++) {
        float ar = a[2 * i], ai = a[2 * i + 1], br = b[2 * i], bi = b[2 * i + 1];
        float tr = ar * br + ai * bi, ti = -ar * bi + ai * br;
        float mag = sqrtf(tr * tr + ti * ti);
        out[2 * i] = tr / mag;
        out[2 * i + 1] = ti / mag;
    }
}

/* magSpectrums / logMagSpectrums (glsBasicOperation.cpp:117-119, :126-128,
 * shader ops 9 and 13): sqrt(re^2 + im^2), log(|sqrt(re^2 + im^2) + offset|). */
void oracle_mag_spectrums(const float *a, float *out, size_t n, int log_mag, float offset) {
    for (size_t i = 0; i < n; i++) {
        float r = a[2 * i], g = a[2 * i + 1];
        float mag = sqrtf(r * r + g * g);
        out[i] = log_mag ? logf(fabsf(mag + offset)) : mag;
    }
}

/* gls::minMaxLoc (glsCV/glsMinMaxLoc.cpp:65-119, :149-200): a strict-compare
 * scan of every row from the FLT_MAX literal of the shader, then a strict
 * scan of the row results -- the first occurrence in row-major order; an
 * element takes part only if it compares below (above) the literal, and
 * when none does the result is the literal at (0, 0).  loc = {x, y}. */
void oracle_min_max_loc(const float *x, int rows, int cols, double *min_val, double *max_val,
                        int *min_loc, int *max_loc) {
    const float lit = 3.402823e+38f;
    float gmin = lit, gmax = -lit;
    int gminx = 0, gminy = 0, gmaxx = 0, gmaxy = 0;
    for (int y = 0; y < rows; y++) {
        float rmin = lit, rmax = -lit;
        int rminx = 0, rmaxx = 0;
        for (int c = 0; c < cols; c++) {
            float d = x[(size_t)y * cols + c];
            if (d < rmin) { rmin = d; rminx = c; }
            if (d > rmax) { rmax = d; rmaxx = c; }
        }
        if (rmin < gmin) { gmin = rmin; gminx = rminx; gminy = y; }
        if (rmax > gmax) { gmax = rmax; gmaxx = rmaxx; gmaxy = y; }
    }
    /* rows that never updated report x = 0 of their own row, as the shader's
     * second pass reads the row's stored location (0 by default) */
    if (min_val) *min_val = gmin;
    if (max_val) *max_val = gmax;
    if (min_loc) { min_loc[0] = gminx; min_loc[1] = gminy; }
    if (max_loc) { max_loc[0] = gmaxx; max_loc[1] = gmaxy; }
}

/* gls::normalize(src, dst, alpha, beta, NORM_MINMAX) (glsCV/glsNormalize.cpp:52-68):
 * scl = (float)(beta - alpha) / (float)(max - min); dst = (float)(alpha - scl*min)
 * + scl * src, the product and the sum each rounded to float. */
void oracle_normalize_minmax(const float *x, float *out, int rows, int cols, double alpha,
                             double beta) {
    double mn, mx;
    oracle_min_max_loc(x, rows, cols, &mn, &mx, 0, 0);
    float scl = (float)(beta - alpha) / (float)(mx - mn);
    float c = (float)(alpha - (double)scl * mn);
    size_t n = (size_t)rows * cols;
    for (size_t i = 0; i < n; i++) {
        float t = scl * x[i];
        out[i] = c + t;
    }
}

int oracle_num_threads(void) {
#ifdef _OPENMP
    return omp_get_max_threads();
#else
    return 1;
#endif
}

void oracle_set_threads(int n) {
#ifdef _OPENMP
    if (n > 0) omp_set_num_threads(n);
#else
    (void)n;
#endif
}
