// tc_fft.cu -- precision form: 1-D line FFTs of length N = N1*N1 (1024 = 32^2,
// 4096 = 64^2) as tensor-core complex matrix products with FP16 hi/lo split
// operands (three products, FP32 accumulate).
//
// Four-step on each line, viewed as an N1 x N1 matrix X[n1][n2] = x[N1 n1 + n2]:
//   A:  Y = F * X                (F[k][n] = e^{-2 pi i k n / N1})
//   B:  Z[k1][n2] = Y[k1][n2] * e^{-2 pi i k1 n2 / N}
//   C:  O = F * Z^T,  X_out[k1 + N1 k2] = O[k2][k1]   (natural order, row-major O)
// Each complex product runs as the real product [Fr -Fi; Fi Fr] (2N1 x 2N1)
// times [Br; Bi] (2N1 x N1) on mma.sync m16n8k16 (f16 x f16 -> f32).  Every
// operand is split v = hi + lo (hi = fp16(v), lo = fp16(v - hi)) after a
// power-of-two block scale that puts the tile's largest magnitude near 2^14,
// and the product accumulates Fhi*Bhi + Fhi*Blo + Flo*Bhi in FP32 -- about 22
// mantissa bits per product, FP32-level error overall.  Stage B is fused into
// stage C's operand build.  F (hi/lo) and the stage-B twiddles are generated
// in FP64 on the host once per context.
#include <cuda_fp16.h>

#include "fft_kernels.cuh"
#include "glsfft_internal.h"
#include "tc_internal.h"

namespace glsfft {

namespace {

constexpr int kTcThreads = 256;

__device__ __forceinline__ unsigned pack2(__half lo_elem, __half hi_elem) {
    return (unsigned)__half_as_ushort(lo_elem) | ((unsigned)__half_as_ushort(hi_elem) << 16);
}

__device__ __forceinline__ void split2(float a, float b, unsigned &hi, unsigned &lo) {
    const __half ah = __float2half_rn(a), bh = __float2half_rn(b);
    const __half al = __float2half_rn(a - __half2float(ah)), bl = __float2half_rn(b - __half2float(bh));
    hi = pack2(ah, bh);
    lo = pack2(al, bl);
}

__device__ __forceinline__ void mma16816(float (&d)[4], const unsigned (&a)[4], unsigned b0,
                                         unsigned b1) {
    asm volatile(
        "mma.sync.aligned.m16n8k16.row.col.f32.f16.f16.f32 {%0,%1,%2,%3}, {%4,%5,%6,%7}, {%8,%9}, "
        "{%0,%1,%2,%3};"
        : "+f"(d[0]), "+f"(d[1]), "+f"(d[2]), "+f"(d[3])
        : "r"(a[0]), "r"(a[1]), "r"(a[2]), "r"(a[3]), "r"(b0), "r"(b1));
}

// Shared-memory layout per block (N1, L lines of N = N1^2 complex):
//   Fh, Fl: 2N1 x (2N1 + 8) halves (row pad keeps A-fragment loads conflict free)
//   X:      L x N float2, natural order (input, later the output)
//   Y:      L x N float2 (stage A result, [k1][n2])
template <int N1>
struct TcLayout {
    static constexpr int N = N1 * N1;
    static constexpr int L = 4096 / N;         // lines per block
    static constexpr int K2 = 2 * N1;          // real-ified K (and M)
    static constexpr int FSTRIDE = K2 + 8;     // halves per F row
    static constexpr size_t F_BYTES = (size_t)K2 * FSTRIDE * 2;
    static constexpr size_t X_BYTES = (size_t)L * N * 8;
    static constexpr size_t SMEM = 2 * F_BYTES + 2 * X_BYTES + 64;
};

// One stage: out[m][n] for all m < 2N1 of this warp's (line, n-block) =
// sum_k A[m][k] * B[k][n], with B built by `bfetch(k, n) -> float`.
template <int N1, class BFetch, class DStore>
__device__ __forceinline__ void tc_stage(const __half *fh, const __half *fl, int nb, BFetch bfetch,
                                         DStore dstore) {
    using Lay = TcLayout<N1>;
    constexpr int MB = Lay::K2 / 16, KB = Lay::K2 / 16;
    const int lane = threadIdx.x & 31, g = lane >> 2, t = lane & 3;
    // hi*hi products and the two correction products accumulate separately:
    // added into the large running sum, the small terms would lose bits to
    // the tensor core's accumulation
    float acc[MB][4], cor[MB][4];
#pragma unroll
    for (int mb = 0; mb < MB; mb++)
#pragma unroll
        for (int q = 0; q < 4; q++) acc[mb][q] = cor[mb][q] = 0.f;
    const int n = nb * 8 + g;
#pragma unroll 1
    for (int kb = 0; kb < KB; kb++) {
        const int k0 = kb * 16 + 2 * t;
        unsigned bh0, bl0, bh1, bl1;
        split2(bfetch(k0, n), bfetch(k0 + 1, n), bh0, bl0);
        split2(bfetch(k0 + 8, n), bfetch(k0 + 9, n), bh1, bl1);
#pragma unroll
        for (int mb = 0; mb < MB; mb++) {
            const int r = mb * 16 + g;
            const __half *ph = fh + r * Lay::FSTRIDE + kb * 16 + 2 * t;
            const __half *pl = fl + r * Lay::FSTRIDE + kb * 16 + 2 * t;
            unsigned ah[4], al[4];
            ah[0] = *reinterpret_cast<const unsigned *>(ph);
            ah[1] = *reinterpret_cast<const unsigned *>(ph + 8 * Lay::FSTRIDE);
            ah[2] = *reinterpret_cast<const unsigned *>(ph + 8);
            ah[3] = *reinterpret_cast<const unsigned *>(ph + 8 * Lay::FSTRIDE + 8);
            al[0] = *reinterpret_cast<const unsigned *>(pl);
            al[1] = *reinterpret_cast<const unsigned *>(pl + 8 * Lay::FSTRIDE);
            al[2] = *reinterpret_cast<const unsigned *>(pl + 8);
            al[3] = *reinterpret_cast<const unsigned *>(pl + 8 * Lay::FSTRIDE + 8);
            mma16816(acc[mb], ah, bh0, bh1);
            mma16816(cor[mb], ah, bl0, bl1);
            mma16816(cor[mb], al, bh0, bh1);
        }
    }
#pragma unroll
    for (int mb = 0; mb < MB; mb++) {
        const int r = mb * 16 + g, c = nb * 8 + 2 * t;
        dstore(r, c, acc[mb][0] + cor[mb][0]);
        dstore(r, c + 1, acc[mb][1] + cor[mb][1]);
        dstore(r + 8, c, acc[mb][2] + cor[mb][2]);
        dstore(r + 8, c + 1, acc[mb][3] + cor[mb][3]);
    }
}

// Largest |re| or |im| of the block's lines -> power-of-two scale putting it
// just under 2^14 (the FP16 split keeps 22 bits relative to that magnitude).
__device__ __forceinline__ float block_scale(float local_max, float *red) {
#pragma unroll
    for (int off = 16; off > 0; off >>= 1) local_max = fmaxf(local_max, __shfl_xor_sync(0xffffffffu, local_max, off));
    if ((threadIdx.x & 31) == 0) red[threadIdx.x >> 5] = local_max;
    __syncthreads();
    float m = 0.f;
    for (int w = 0; w < kTcThreads / 32; w++) m = fmaxf(m, red[w]);
    __syncthreads();
    if (!(m > 0.f) || !isfinite(m)) return 1.0f;
    int e;
    frexpf(m, &e);  // m = f * 2^e, 0.5 <= f < 1
    return ldexpf(1.0f, 14 - e);
}

// Lines of a launch: rows (stride 1, `LINES` consecutive rows per block) or
// columns (stride cols, `LINES` adjacent columns per block); blockIdx.y = image.
template <int N1, bool ROWS>
__global__ void __launch_bounds__(kTcThreads) tc_lines_kernel(PassArgs a, const __half *g_fh,
                                                               const __half *g_fl,
                                                               const float2 *g_tw) {
    using Lay = TcLayout<N1>;
    constexpr int N = Lay::N, L = Lay::L;
    extern __shared__ __align__(16) unsigned char tc_smem[];
    __half *fh = reinterpret_cast<__half *>(tc_smem);
    __half *fl = fh + Lay::K2 * Lay::FSTRIDE;
    float2 *X = reinterpret_cast<float2 *>(tc_smem + 2 * Lay::F_BYTES);
    float2 *Y = X + L * N;
    float *red = reinterpret_cast<float *>(Y + L * N);

    const float2 *in = static_cast<const float2 *>(image_in(a, blockIdx.y));
    float2 *out = static_cast<float2 *>(image_out(a, blockIdx.y));
    const int cols = a.cols;
    const int line0 = blockIdx.x * L;
    const int nlines = ROWS ? a.rows : cols;
    const bool cin = a.flags & PF_CONJ_IN, cout = a.flags & PF_CONJ_OUT;

    // F hi/lo into shared memory
    for (int i = threadIdx.x; i < Lay::K2 * Lay::FSTRIDE / 2; i += kTcThreads) {
        reinterpret_cast<unsigned *>(fh)[i] = reinterpret_cast<const unsigned *>(g_fh)[i];
        reinterpret_cast<unsigned *>(fl)[i] = reinterpret_cast<const unsigned *>(g_fl)[i];
    }
    // the block's lines, natural order
    float lmax = 0.f;
    for (int i = threadIdx.x; i < L * N; i += kTcThreads) {
        const int l = ROWS ? i / N : i % L, p = ROWS ? i % N : i / L;
        const int line = line0 + l;
        float2 v = make_float2(0.f, 0.f);
        if (line < nlines) v = ROWS ? in[(size_t)line * N + p] : in[(size_t)p * cols + line];
        if (cin) v.y = -v.y;
        X[l * N + p] = v;
        lmax = fmaxf(lmax, fmaxf(fabsf(v.x), fabsf(v.y)));
    }
    __syncthreads();
    const float sA = block_scale(lmax, red);
    const float sC = sA / (float)N1;
    const int warp = threadIdx.x >> 5;
    constexpr int TASKS = L * (N1 / 8);  // (line, n-block) pairs per stage

    // stage A: Y = F * X  (B[k][n] = X[k mod N1][n], real rows then imaginary)
    for (int task = warp; task < TASKS; task += kTcThreads / 32) {
        const int l = task / (N1 / 8), nb = task % (N1 / 8);
        const float2 *xl = X + l * N;
        float2 *yl = Y + l * N;
        tc_stage<N1>(
            fh, fl, nb,
            [&](int k, int n) {
                const float2 v = xl[(k & (N1 - 1)) * N1 + n];
                return (k < N1 ? v.x : v.y) * sA;
            },
            [&](int m, int n, float v) {
                float *dst = reinterpret_cast<float *>(yl + (m & (N1 - 1)) * N1 + n);
                dst[m < N1 ? 0 : 1] = v / sA;
            });
    }
    __syncthreads();
    // stage B (twiddle) fused into stage C: O = F * Z^T, B[k][n] = Z[n][k mod N1]
    for (int task = warp; task < TASKS; task += kTcThreads / 32) {
        const int l = task / (N1 / 8), nb = task % (N1 / 8);
        const float2 *yl = Y + l * N;
        float2 *ol = X + l * N;
        tc_stage<N1>(
            fh, fl, nb,
            [&](int k, int n) {
                const int n2 = k & (N1 - 1);
                const float2 y = yl[n * N1 + n2];
                const float2 w = __ldg(g_tw + n * N1 + n2);
                const float z = k < N1 ? y.x * w.x - y.y * w.y : y.x * w.y + y.y * w.x;
                return z * sC;
            },
            [&](int m, int n, float v) {
                // O[k2][k1] with k2 = m mod N1, k1 = n  ->  X_out[k1 + N1 k2]
                float *dst = reinterpret_cast<float *>(ol + (m & (N1 - 1)) * N1 + n);
                dst[m < N1 ? 0 : 1] = v / sC;
            });
    }
    __syncthreads();
    // store (scale, conj, half swap along the line)
    const float s = a.scale;
    const bool shift = a.flags & (ROWS ? PF_SHIFT_COLS : PF_SHIFT_ROWS);
    for (int i = threadIdx.x; i < L * N; i += kTcThreads) {
        const int l = ROWS ? i / N : i % L, p = ROWS ? i % N : i / L;
        const int line = line0 + l;
        if (line >= nlines) continue;
        float2 v = X[l * N + p];
        v.x *= s;
        v.y *= cout ? -s : s;
        const int op = shift ? (p + N / 2) & (N - 1) : p;
        if (ROWS) out[(size_t)line * N + op] = v;
        else out[(size_t)op * cols + line] = v;
    }
}

template <int N1, bool ROWS>
cudaError_t tc_launch(const PassArgs &a, const TcTables &t, int images, cudaStream_t s) {
    using Lay = TcLayout<N1>;
    auto kern = tc_lines_kernel<N1, ROWS>;
    const cudaError_t e = smem_opt_in(reinterpret_cast<const void *>(kern), Lay::SMEM);
    if (e != cudaSuccess) return e;
    const int nlines = ROWS ? a.rows : a.cols;
    dim3 grid((nlines + Lay::L - 1) / Lay::L, images);
    const __half *fh = N1 == 32 ? t.f32_hi : t.f64_hi;
    const __half *fl = N1 == 32 ? t.f32_lo : t.f64_lo;
    const float2 *tw = N1 == 32 ? t.tw1024 : t.tw4096;
    kern<<<grid, kTcThreads, Lay::SMEM, s>>>(a, fh, fl, tw);
    return cudaGetLastError();
}

}  // namespace

cudaError_t launch_tc_lines(int n, bool rows, const PassArgs &a, const TcTables &t, int images,
                            cudaStream_t s) {
    if (n == 1024 || n == 4096) return launch_tc5_lines(n, rows, a, t, images, s);
    if (n == 4096) return rows ? tc_launch<64, true>(a, t, images, s) : tc_launch<64, false>(a, t, images, s);
    return cudaErrorInvalidValue;
}

size_t tc_f_row_halves(int n1) { return (size_t)(2 * n1 + 8); }

}  // namespace glsfft
