// fft_device.cuh -- device building blocks of the GB300 FFT path.
//
// One power-of-two FFT "line" (a row or a column of a CV_32FC2 image) is
// computed by T = N/E threads, each holding E complex values in registers.
// Passes are Stockham autosort radix-R steps (R in {2,4,8,16}, balanced so
// that ceil(log2 N / 4) passes suffice).  The first pass takes its operands
// straight from the global load, the last pass leaves results in the same
// registers in natural order for the global store, and the passes in between
// exchange through shared memory, so a line costs one global read and one
// global write.  This replaces the reference's one-draw-per-radix-4-pass
// fragment shader (glsCV/glsFft.cpp:203-343) and its ping-pong textures
// (glsFft.cpp:528-532).
//
// Register slot m of thread t always holds line position t + m*T on entry to
// a pass; in a pass with radix R and span Ns, butterfly j = t + s*T
// (s < E/R) reads slots s + r*E/R (positions j + r*N/R), twiddles by
// w_N^{(j mod Ns) * r * N/(Ns*R)}, runs an R-point DFT and writes positions
// (j/Ns)*Ns*R + (j mod Ns) + r*Ns.
#pragma once
#include <cuda_runtime.h>
#include <stdint.h>

#include "glsfft_internal.h"

namespace glsfft {

// ------------------------------------------------------------ complex helpers
// Complex add / subtract as one packed FP32x2 instruction (sm_100 family);
// each lane rounds exactly like the scalar operation.
__device__ __forceinline__ unsigned long long f2_bits(float2 a) {
    return *reinterpret_cast<unsigned long long *>(&a);
}
__device__ __forceinline__ float2 bits_f2(unsigned long long u) {
    return *reinterpret_cast<float2 *>(&u);
}
__device__ __forceinline__ float2 cadd(float2 a, float2 b) {
    unsigned long long d;
    asm("add.rn.f32x2 %0, %1, %2;" : "=l"(d) : "l"(f2_bits(a)), "l"(f2_bits(b)));
    return bits_f2(d);
}
__device__ __forceinline__ float2 csub(float2 a, float2 b) {
    unsigned long long d;
    asm("sub.rn.f32x2 %0, %1, %2;" : "=l"(d) : "l"(f2_bits(a)), "l"(f2_bits(b)));
    return bits_f2(d);
}
// a + (s.x * b.y, s.y * b.x) for s = (+-1, +-1): a +- i*b in one packed FMA
// (the products by +-1 are exact, so each lane equals the scalar add/sub)
__device__ __forceinline__ float2 cadd_swapped(float2 a, float2 b, float2 s) {
    unsigned long long d;
    const float2 bs = make_float2(b.y, b.x);
    asm("fma.rn.f32x2 %0, %1, %2, %3;" : "=l"(d) : "l"(f2_bits(bs)), "l"(f2_bits(s)), "l"(f2_bits(a)));
    return bits_f2(d);
}
// (a.x * sx, a.y * sy) as one packed multiply
__device__ __forceinline__ float2 cmul_re(float2 a, float sx, float sy) {
    unsigned long long d;
    asm("mul.rn.f32x2 %0, %1, %2;" : "=l"(d) : "l"(f2_bits(a)), "l"(f2_bits(make_float2(sx, sy))));
    return bits_f2(d);
}
// Complex product with explicit fused multiply-adds: every kernel that
// inlines it rounds the same way, whatever contraction the compiler would
// choose, so the batch, pass and plain kernels give bit-identical lines.
__device__ __forceinline__ float2 cmul(float2 a, float2 b) {
    return make_float2(__fmaf_rn(a.x, b.x, -__fmul_rn(a.y, b.y)),
                       __fmaf_rn(a.x, b.y, __fmul_rn(a.y, b.x)));
}
__device__ __forceinline__ float2 cconj(float2 a) { return make_float2(a.x, -a.y); }
__device__ __forceinline__ float2 cscale(float2 a, float s) { return make_float2(a.x * s, a.y * s); }

// --------------------------------------------------------- radix schedule
// mb = log2 of the largest radix allowed (4: radix <= 16, the default; 3:
// radix <= 8, one more pass for most lengths but half the registers).
__host__ __device__ constexpr int ilog2c(int n) { return n <= 1 ? 0 : 1 + ilog2c(n >> 1); }
__host__ __device__ constexpr int num_passes(int n, int mb = 4) {
    return ilog2c(n) == 0 ? 0 : (ilog2c(n) <= mb ? 1 : (ilog2c(n) + mb - 1) / mb);
}
__host__ __device__ constexpr int pass_bits(int n, int p, int mb = 4) {
    return ilog2c(n) / num_passes(n, mb) + (p < ilog2c(n) % num_passes(n, mb) ? 1 : 0);
}
__host__ __device__ constexpr int pass_radix(int n, int p, int mb = 4) {
    return 1 << pass_bits(n, p, mb);
}
__host__ __device__ constexpr int pass_span(int n, int p, int mb = 4) {
    return p == 0 ? 1 : pass_span(n, p - 1, mb) * pass_radix(n, p - 1, mb);
}
__host__ __device__ constexpr int max_radix(int n, int mb = 4) {
    return num_passes(n, mb) == 0 ? 1 : pass_radix(n, 0, mb);
}

// ------------------------------------------- multiply by w_R^K = e^{-2 pi i K/R}
// Exact special cases for multiples of pi/4; cos/sin(pi/8) constants otherwise.
template <int K, int R>
__device__ __forceinline__ float2 wmul(float2 v) {
    constexpr int k16 = ((K % R) + R) % R * (16 / R);
    constexpr float S = 0.70710678118654752440f;  // sqrt(1/2)
    constexpr float C1 = 0.92387953251128675613f; // cos(pi/8)
    constexpr float S1 = 0.38268343236508977173f; // sin(pi/8)
    if constexpr (k16 == 0) return v;
    else if constexpr (k16 == 4) return make_float2(v.y, -v.x);
    else if constexpr (k16 == 8) return make_float2(-v.x, -v.y);
    else if constexpr (k16 == 12) return make_float2(-v.y, v.x);
    // odd multiples of pi/4: the sum and difference of the components, then
    // one packed multiply (each lane rounds like the scalar expression)
    else if constexpr (k16 == 2) return cmul_re(cadd_swapped(v, v, make_float2(1.f, -1.f)), S, S);
    else if constexpr (k16 == 6) {
        const float2 t = cadd_swapped(v, v, make_float2(1.f, -1.f));  // (x+y, y-x)
        return cmul_re(make_float2(t.y, t.x), S, -S);
    } else if constexpr (k16 == 10) {
        const float2 t = cadd_swapped(v, v, make_float2(-1.f, 1.f));  // (x-y, y+x)
        return cmul_re(make_float2(t.y, t.x), -S, S);
    } else if constexpr (k16 == 14) return cmul_re(cadd_swapped(v, v, make_float2(-1.f, 1.f)), S, S);
    else {
        // odd multiples of pi/8: e^{-i k pi/8}
        constexpr float c = (k16 == 1 || k16 == 15) ? C1 : (k16 == 3 || k16 == 13) ? S1
                          : (k16 == 5 || k16 == 11) ? -S1 : -C1;
        constexpr float s = (k16 == 1 || k16 == 7) ? -S1 : (k16 == 3 || k16 == 5) ? -C1
                          : (k16 == 9 || k16 == 15) ? S1 : C1;
        return make_float2(__fmaf_rn(v.x, c, -__fmul_rn(v.y, s)), __fmaf_rn(v.x, s, __fmul_rn(v.y, c)));
    }
}

// ------------------------------------------------ R-point DFTs in registers
// In place, natural-order output, forward sign.
template <int R> struct Dft;
template <> struct Dft<1> { __device__ __forceinline__ static void run(float2 *) {} };
template <> struct Dft<2> {
    __device__ __forceinline__ static void run(float2 *v) {
        float2 a = v[0], b = v[1];
        v[0] = cadd(a, b);
        v[1] = csub(a, b);
    }
};
template <> struct Dft<4> {
    __device__ __forceinline__ static void run(float2 *v) {
        float2 apc = cadd(v[0], v[2]), amc = csub(v[0], v[2]);
        float2 bpd = cadd(v[1], v[3]), bmd = csub(v[1], v[3]);
        v[0] = cadd(apc, bpd);
        v[2] = csub(apc, bpd);
        v[1] = cadd_swapped(amc, bmd, make_float2(1.f, -1.f));  // amc - i*bmd
        v[3] = cadd_swapped(amc, bmd, make_float2(-1.f, 1.f));  // amc + i*bmd
    }
};
template <> struct Dft<8> {
    __device__ __forceinline__ static void run(float2 *v) {
        float2 e[4] = {v[0], v[2], v[4], v[6]};
        float2 o[4] = {v[1], v[3], v[5], v[7]};
        Dft<4>::run(e);
        Dft<4>::run(o);
        o[1] = wmul<1, 8>(o[1]);
        o[2] = wmul<2, 8>(o[2]);
        o[3] = wmul<3, 8>(o[3]);
#pragma unroll
        for (int k = 0; k < 4; k++) {
            v[k] = cadd(e[k], o[k]);
            v[k + 4] = csub(e[k], o[k]);
        }
    }
};
template <> struct Dft<16> {
    __device__ __forceinline__ static void run(float2 *v) {
        float2 a0[4] = {v[0], v[4], v[8], v[12]};
        float2 a1[4] = {v[1], v[5], v[9], v[13]};
        float2 a2[4] = {v[2], v[6], v[10], v[14]};
        float2 a3[4] = {v[3], v[7], v[11], v[15]};
        Dft<4>::run(a0);
        Dft<4>::run(a1);
        Dft<4>::run(a2);
        Dft<4>::run(a3);
        a1[1] = wmul<1, 16>(a1[1]); a1[2] = wmul<2, 16>(a1[2]); a1[3] = wmul<3, 16>(a1[3]);
        a2[1] = wmul<2, 16>(a2[1]); a2[2] = wmul<4, 16>(a2[2]); a2[3] = wmul<6, 16>(a2[3]);
        a3[1] = wmul<3, 16>(a3[1]); a3[2] = wmul<6, 16>(a3[2]); a3[3] = wmul<9, 16>(a3[3]);
#pragma unroll
        for (int k1 = 0; k1 < 4; k1++) {
            float2 b[4] = {a0[k1], a1[k1], a2[k1], a3[k1]};
            Dft<4>::run(b);
            v[k1] = b[0];
            v[k1 + 4] = b[1];
            v[k1 + 8] = b[2];
            v[k1 + 12] = b[3];
        }
    }
};

// ------------------------------------------------------- the line engine
// Barrier policies for the exchanges: the whole block, or only the 256
// compute threads of a warp-specialised block (named barrier 1).
struct SyncBlock {
    __device__ __forceinline__ void operator()() const { __syncthreads(); }
};
struct SyncCompute256 {
    __device__ __forceinline__ void operator()() const {
        asm volatile("bar.sync 1, 256;" ::: "memory");
    }
};

// ------------------------------------------------------ twiddle sources
// Row k of the table of a pass with radix R and span L = Ns*R: w^(R/2) in
// w[0] (R > 2) and w^1..w^(R/2-1) in w[1..], w = e^{-2 pi i k / L}; for
// R = 2, w[0] = w^1.  From the global tables (tw_offset layout):
template <int N, int MB, int P_, int R, int L>
__device__ __forceinline__ void tw_row(const float2 *__restrict__ tw, int k, float2 (&w)[R / 2]) {
    const float2 *wt = tw + tw_offset(R, L) + k * R;
    if constexpr (R == 2) {
        w[0] = __ldg(wt);
    } else {
        const float4 *w4 = reinterpret_cast<const float4 *>(wt);
#pragma unroll
        for (int h = 0; h < R / 4; h++) {
            const float4 q = __ldg(w4 + h);
            w[2 * h] = make_float2(q.x, q.y);
            w[2 * h + 1] = make_float2(q.z, q.w);
        }
    }
}

// A line's tables for passes 1..P-1 copied into shared memory.  Pass p's
// table (L_p / R_p rows of R_p / 4 float4 vectors) is stored vector-major,
// [vector h][row k], so the consecutive butterflies of a warp read
// consecutive 16-byte words.  Needs R_p >= 4 for every p >= 1.
__host__ __device__ constexpr int tw_smem_offset4(int n, int p, int mb) {
    return p <= 1 ? 0
                  : tw_smem_offset4(n, p - 1, mb) + pass_span(n, p - 1, mb) * pass_radix(n, p - 1, mb) / 4;
}
__host__ __device__ constexpr int tw_smem_float4(int n, int mb = 4) {
    return num_passes(n, mb) <= 1 ? 0 : tw_smem_offset4(n, num_passes(n, mb), mb);
}
__host__ __device__ constexpr bool tw_smem_ok_from(int n, int p, int mb) {
    return p >= num_passes(n, mb) ? true : (pass_radix(n, p, mb) >= 4 && tw_smem_ok_from(n, p + 1, mb));
}
__host__ __device__ constexpr bool tw_smem_ok(int n, int mb = 4) { return tw_smem_ok_from(n, 1, mb); }

template <int N, int MB = 4>
struct SmemTw {
    const float4 *base;  // shared memory, tw_smem_float4(N, MB) vectors
};

template <int N, int MB, int P_, int R, int L>
__device__ __forceinline__ void tw_row(const SmemTw<N, MB> &tw, int k, float2 (&w)[R / 2]) {
    static_assert(R >= 4, "shared-memory twiddles need radix >= 4");
    constexpr int rows = L / R;
    const float4 *w4 = tw.base + tw_smem_offset4(N, P_, MB) + k;
#pragma unroll
    for (int h = 0; h < R / 4; h++) {
        const float4 q = w4[h * rows];
        w[2 * h] = make_float2(q.x, q.y);
        w[2 * h + 1] = make_float2(q.z, q.w);
    }
}

// Copy a line's tables from the global tables into `dst` (shared memory);
// threads tid = 0..nthreads-1 share the work.
template <int N, int MB, int p>
__device__ __forceinline__ void tw_fill_pass(float4 *dst, const float2 *__restrict__ tw, int tid,
                                             int nthreads) {
    if constexpr (p < num_passes(N, MB)) {
        constexpr int R = pass_radix(N, p, MB), L = pass_span(N, p, MB) * R, rows = L / R;
        const float4 *src = reinterpret_cast<const float4 *>(tw + tw_offset(R, L));
        float4 *d = dst + tw_smem_offset4(N, p, MB);
        for (int i = tid; i < rows * (R / 4); i += nthreads) {
            const int k = i % rows, h = i / rows;
            d[h * rows + k] = __ldg(src + k * (R / 2) + h);
        }
        tw_fill_pass<N, MB, p + 1>(dst, tw, tid, nthreads);
    }
}
template <int N, int MB = 4>
__device__ __forceinline__ void tw_fill_smem(float4 *dst, const float2 *__restrict__ tw, int tid,
                                             int nthreads) {
    static_assert(tw_smem_ok(N, MB), "a pass with radix 2 has no shared-memory table");
    tw_fill_pass<N, MB, 1>(dst, tw, tid, nthreads);
}

// Shared-memory accessors map a line position to a padded slot: the linear
// index i (position * KW + column) gets one pad per 16, slot = i + i/16.
// Strided<Sm, DELTA, COUNT> tells whether COUNT accesses DELTA positions
// apart from a base are a fixed slot step apart (so one address and
// compile-time offsets serve them all): true when the linear step is a
// multiple of 16, or when all COUNT accesses fall inside one 16-slot block
// (the base is then aligned to DELTA*COUNT*KW, as every caller's base is).
template <class Sm, int DELTA, int COUNT>
struct Strided {
    static constexpr int LIN = DELTA * Sm::KW;
    static constexpr bool by_block = (LIN % 16) == 0;
    static constexpr bool in_block = LIN * COUNT <= 16;
    static constexpr bool affine = by_block || in_block;
    static constexpr int STEP = by_block ? LIN + LIN / 16 : LIN;
};

// Sm: shared-memory accessor for this thread's line: at(pos) -> float2*
// (one exchange of complex values, KW as above), or, with Sm::kSplit,
// at<X>(pos) -> float* for the exchange after pass X (the exchange runs
// twice through a buffer half the size, real parts then imaginary parts;
// each exchange may pad differently, as its stores and loads are its own).
// tw: the per-pass twiddle tables above.
template <int N, int E, class Sync = SyncBlock, int MB = 4>
struct LineFft {
    static_assert((N & (N - 1)) == 0 && N >= 1 && N <= 8192, "N must be a power of two");
    static_assert(N == 1 || (N % E) == 0, "E must divide N");
    static constexpr int T = (N >= E) ? N / E : 1;
    static constexpr int P = num_passes(N, MB);

    // Tw: const float2 * (the global tables) or SmemTw<N, MB> (a copy in
    // shared memory).  When run() returns, other threads may still be
    // reading the exchange buffer: sync before writing it again.
    template <class Sm, class Tw>
    __device__ __forceinline__ static void run(float2 (&x)[E], int t, Sm sm, Tw tw) {
        pass<0>(x, t, sm, tw);
    }

    template <int p, class Sm, class Tw>
    __device__ __forceinline__ static void pass(float2 (&x)[E], int t, Sm sm, Tw tw) {
        if constexpr (p < P) {
            [[maybe_unused]] const Sync sync{};
            constexpr int R = pass_radix(N, p, MB);
            constexpr int Ns = pass_span(N, p, MB);
            constexpr int S = E / R;
            constexpr bool last = (Ns * R == N);
            static_assert(E % R == 0, "E must be a multiple of every radix");
#pragma unroll
            for (int s = 0; s < S; s++) {
                const int j = t + s * T;
                float2 v[R];
#pragma unroll
                for (int r = 0; r < R; r++) v[r] = x[s + r * S];
                if constexpr (Ns > 1) {
                    // w^0..w^(R/2-1) come from the table (R/4 16-byte loads);
                    // w^(R/2+r) = w^(R/2) * w^r, one extra rounding, halves
                    // the twiddle loads (entry R/2 is stored in slot 0, whose
                    // value w^0 = 1 is never needed)
                    const int k = j & (Ns - 1);
                    float2 w[R / 2];
                    tw_row<N, MB, p, R, Ns * R>(tw, k, w);
                    if constexpr (R == 2) {
                        v[1] = cmul(v[1], w[0]);
                    } else {
                        const float2 wh = w[0];  // w^(R/2)
#pragma unroll
                        for (int r = 1; r < R / 2; r++) {
                            v[r] = cmul(v[r], w[r]);
                            v[r + R / 2] = cmul(v[r + R / 2], cmul(wh, w[r]));
                        }
                        v[R / 2] = cmul(v[R / 2], wh);
                    }
                }
                Dft<R>::run(v);
                if constexpr (last || Sm::kSplit) {
#pragma unroll
                    for (int r = 0; r < R; r++) x[s + r * S] = v[r];
                } else {
                    const int d = (j / Ns) * Ns * R + (j & (Ns - 1));
                    using WS = Strided<Sm, Ns, R>;
                    if constexpr (WS::affine) {
                        float2 *o = sm.at(d);
#pragma unroll
                        for (int r = 0; r < R; r++) o[r * WS::STEP] = v[r];
                    } else {
#pragma unroll
                        for (int r = 0; r < R; r++) *sm.at(d + r * Ns) = v[r];
                    }
                }
            }
            if constexpr (!last && Sm::kSplit) {
                exchange_half<p, 0>(x, t, sm);
                exchange_half<p, 1>(x, t, sm);
                pass<p + 1>(x, t, sm, tw);
            } else if constexpr (!last) {
                sync();
                using RS = Strided<Sm, T, E>;
                if constexpr (RS::affine) {
                    const float2 *in = sm.at(t);
#pragma unroll
                    for (int m = 0; m < E; m++) x[m] = in[m * RS::STEP];
                } else {
#pragma unroll
                    for (int m = 0; m < E; m++) x[m] = *sm.at(t + m * T);
                }
                // the next exchange overwrites the buffer; after the last one
                // the caller syncs before it writes the buffer again
                if constexpr (p + 2 < P) sync();
                pass<p + 1>(x, t, sm, tw);
            }
        }
    }

    // One component (H = 0: real, 1: imaginary) of the exchange after pass
    // p, through a float buffer: the butterfly outputs, still in x in their
    // pass order, go to their Stockham positions; the reads bring back
    // positions t + m*T.  The other component's registers are untouched, so
    // the second half still sees the pre-exchange order.
    template <int p, int H, class Sm>
    __device__ __forceinline__ static void exchange_half(float2 (&x)[E], int t, Sm sm) {
        const Sync sync{};
        constexpr int R = pass_radix(N, p, MB);
        constexpr int Ns = pass_span(N, p, MB);
        constexpr int S = E / R;
#pragma unroll
        for (int s = 0; s < S; s++) {
            const int j = t + s * T;
            const int d = (j / Ns) * Ns * R + (j & (Ns - 1));
#pragma unroll
            for (int r = 0; r < R; r++)
                *sm.template at<p>(d + r * Ns) = H ? x[s + r * S].y : x[s + r * S].x;
        }
        sync();
#pragma unroll
        for (int m = 0; m < E; m++) {
            const float v = *sm.template at<p>(t + m * T);
            if constexpr (H == 0) x[m].x = v;
            else x[m].y = v;
        }
        // the second half, or the next exchange, overwrites the buffer
        if constexpr (H == 0 || p + 2 < P) sync();
    }
};

// --------------------------------------------------- argmax key (first max)
// Max value wins; equal values resolve to the smaller row-major index, which
// is the first occurrence the reference's strict '>' scans keep
// (glsCV/glsMinMaxLoc.cpp:91, :109).  NaN and values <= -FLT_MAX never win.
__device__ __forceinline__ unsigned long long argmax_key(float v, unsigned idx) {
    if (!(v > -3.402823466e+38f)) return 0ull;
    unsigned b = __float_as_uint(v);
    unsigned o = (b & 0x80000000u) ? ~b : (b | 0x80000000u);
    return ((unsigned long long)o << 32) | (unsigned long long)(0xFFFFFFFFu - idx);
}
__device__ __forceinline__ float key_value(unsigned long long key) {
    unsigned o = (unsigned)(key >> 32);
    unsigned b = (o & 0x80000000u) ? (o & 0x7FFFFFFFu) : ~o;
    return __uint_as_float(b);
}
__device__ __forceinline__ unsigned key_index(unsigned long long key) {
    return 0xFFFFFFFFu - (unsigned)(key & 0xFFFFFFFFull);
}

// Block-wide max of keys; thread 0 issues one atomicMax.  `red` needs
// blockDim.x/32 entries of shared memory.
__device__ __forceinline__ void block_argmax_commit(unsigned long long key,
                                                    unsigned long long *red,
                                                    unsigned long long *dst) {
#pragma unroll
    for (int off = 16; off > 0; off >>= 1) {
        unsigned long long o = __shfl_xor_sync(0xffffffffu, key, off);
        key = o > key ? o : key;
    }
    const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
    if (lane == 0) red[warp] = key;
    __syncthreads();
    if (threadIdx.x == 0) {
        unsigned long long best = 0;
        for (int w = 0; w < (int)(blockDim.x >> 5); w++) best = red[w] > best ? red[w] : best;
        if (best) atomicMax(dst, best);
    }
}

}  // namespace glsfft
