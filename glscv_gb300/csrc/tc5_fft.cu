// tc5_fft.cu -- precision form on the fifth-generation tensor cores: line FFTs
// of N = N1^2 points (1024 = 32^2, 4096 = 64^2; rows or columns of CV_32FC2
// images) as a four-step whose two DFT stages are tcgen05 matrix products with
// FP16 hi/lo split operands (hi*hi into one FP32 accumulator, hi*lo + lo*hi
// into a second, both in tensor memory), so the result keeps FP32-level error.
//
// A line x is the N1 x N1 matrix X[n1][n2] = x[N1 n1 + n2]:
//   stage A  Y[k1][n2] = sum_n1 x[N1 n1 + n2] e^{-2 pi i n1 k1 / N1}
//   stage B  Y'[k1][n2] = Y[k1][n2] e^{-2 pi i k1 n2 / N}
//   stage C  out[k1 + N1 k2] = sum_n2 Y'[k1][n2] e^{-2 pi i n2 k2 / N1}
// Each DFT stage is one GEMM over a tile of 128 / N1 lines: 128 rows (line,
// n2) resp. (line, k1), K = 2 N1 (real parts then imaginary parts of the N1
// inputs), N = 2 N1 outputs (real then imaginary), against the real form of
// the N1-point DFT matrix.  N1 = 32: one 64 x 64 B operand [C S; -S C];
// N1 = 64: its 64 x 64 blocks C, S and -S, each product split by output half.
// A thread owns one GEMM row and 32 of its complex values (N1 = 64: two
// threads per row): it loads its inputs, splits them after a power-of-two
// scale (hi = fp16(v), lo = fp16(v - hi)) into the A operands in shared memory
// (K-major, 128-byte swizzle), and reads its part of the accumulator row back
// from tensor memory.  Stage B and the stage-C operand build (a transposing
// write, conflict-free in the swizzled layout) happen between the products.
// One elected thread issues the MMAs; completion arrives on an mbarrier whose
// waits are bounded (GLSFFT_ERROR_TIMEOUT into the status word on expiry).
#include <cuda_fp16.h>

#include "fft_kernels.cuh"
#include "glsfft.h"
#include "glsfft_internal.h"
#include "tc5_device.cuh"
#include "tc_internal.h"

namespace glsfft {

namespace {

constexpr long long kT5WaitNs = 2000000000ll;
constexpr unsigned kT5OpBlock = 128 * 128;  // a 128-row x 64-half operand block

// Shapes per N1: threads (one per GEMM row and output half), lines per tile,
// A operand bytes (one split), B operand bytes (one split), TMEM columns,
// resident blocks per SM.
template <int N1>
struct T5 {
    static constexpr int N = N1 * N1;
    static constexpr int THREADS = 128 * (N1 / 32);
    static constexpr int LINES = 128 / N1;
    static constexpr unsigned OP = kT5OpBlock * (N1 / 32);         // K = 2 N1 halves
    static constexpr unsigned DFT = N1 == 32 ? 64 * 128 : 3 * 64 * 128;  // [C S;-S C] or C,S,-S
    static constexpr int TCOLS = 4 * N1;                            // D1 re, im; D2 re, im
    static constexpr int BLOCKS = N1 == 32 ? 4 : 2;
    // operands, then the mbarrier, TMEM slot and reduction scratch; the
    // dynamic shared memory must start 1024-byte aligned (checked in the kernel)
    static constexpr size_t SMEM = 2 * OP + 2 * DFT + 64 + 4 * 64;
};

// power of two putting m just under 2^14 (the FP16 split then keeps 22 bits
// of every value without reaching FP16's range limit in the products)
__device__ __forceinline__ float pow2_scale(float m) {
    if (!(m > 0.f) || !isfinite(m)) return 1.0f;
    int e;
    frexpf(m, &e);  // m = f * 2^e, 0.5 <= f < 1
    return ldexpf(1.0f, 14 - e);
}

__device__ __forceinline__ void split_half(float v, __half &h, __half &l) {
    h = __float2half_rn(v);
    l = __float2half_rn(v - __half2float(h));  // v - h is exact in FP32
}

__device__ __forceinline__ uint4 pack8(const __half (&h)[8]) {
    uint4 q;
    q.x = (unsigned)__half_as_ushort(h[0]) | ((unsigned)__half_as_ushort(h[1]) << 16);
    q.y = (unsigned)__half_as_ushort(h[2]) | ((unsigned)__half_as_ushort(h[3]) << 16);
    q.z = (unsigned)__half_as_ushort(h[4]) | ((unsigned)__half_as_ushort(h[5]) << 16);
    q.w = (unsigned)__half_as_ushort(h[6]) | ((unsigned)__half_as_ushort(h[7]) << 16);
    return q;
}

// byte offset of A-operand element (row r, k) with K = 2 N1: 64-wide blocks
// of 128 rows, each 128-byte swizzled
__device__ __forceinline__ unsigned op_offset(unsigned r, unsigned k) {
    return (k >> 6) * kT5OpBlock + sw128_offset(r, k & 63u);
}

// The products of one DFT stage.  D1 = Ahi Bhi, D2 = Ahi Blo + Alo Bhi.
// N1 = 32: B = [C S; -S C] (64 x 64), D1 in TMEM columns 0-63 (re k1, im k1),
// D2 in 64-127; K = 64 in four steps of 16.
// N1 = 64: A = [A_re | A_im] (two 64-wide K blocks), B blocks C, S, -S;
// re out = A_re C + A_im S, im out = A_im C + A_re (-S); D1 re / im in
// columns 0-63 / 64-127, D2 re / im in 128-191 / 192-255.
template <int N1>
__device__ __forceinline__ void t5_products(unsigned a_hi, unsigned a_lo, unsigned b_hi,
                                            unsigned b_lo, unsigned tmem) {
    if constexpr (N1 == 32) {
        constexpr uint32_t idesc = umma_idesc_f16(128, 64);
#pragma unroll
        for (int kk = 0; kk < 4; kk++) {
            const uint64_t ah = umma_desc_sw128(a_hi + 32 * kk), al = umma_desc_sw128(a_lo + 32 * kk);
            const uint64_t bh = umma_desc_sw128(b_hi + 32 * kk), bl = umma_desc_sw128(b_lo + 32 * kk);
            umma_f16(tmem, ah, bh, idesc, kk > 0);
            umma_f16(tmem + 64, ah, bl, idesc, kk > 0);
            umma_f16(tmem + 64, al, bh, idesc, 1);
        }
    } else {
        constexpr uint32_t idesc = umma_idesc_f16(128, 64);
        constexpr unsigned BLK = 64 * 128;  // one 64 x 64-half B block
#pragma unroll
        for (int kk = 0; kk < 4; kk++) {
            const unsigned o = 32 * kk;
            const uint64_t reh = umma_desc_sw128(a_hi + o), rel = umma_desc_sw128(a_lo + o);
            const uint64_t imh = umma_desc_sw128(a_hi + kT5OpBlock + o);
            const uint64_t iml = umma_desc_sw128(a_lo + kT5OpBlock + o);
            const uint64_t ch = umma_desc_sw128(b_hi + o), cl = umma_desc_sw128(b_lo + o);
            const uint64_t sh = umma_desc_sw128(b_hi + BLK + o), sl = umma_desc_sw128(b_lo + BLK + o);
            const uint64_t nh = umma_desc_sw128(b_hi + 2 * BLK + o);
            const uint64_t nl = umma_desc_sw128(b_lo + 2 * BLK + o);
            const unsigned first = kk > 0;
            umma_f16(tmem, reh, ch, idesc, first);         // D1 re
            umma_f16(tmem, imh, sh, idesc, 1);
            umma_f16(tmem + 64, imh, ch, idesc, first);    // D1 im
            umma_f16(tmem + 64, reh, nh, idesc, 1);
            umma_f16(tmem + 128, reh, cl, idesc, first);   // D2 re
            umma_f16(tmem + 128, rel, ch, idesc, 1);
            umma_f16(tmem + 128, imh, sl, idesc, 1);
            umma_f16(tmem + 128, iml, sh, idesc, 1);
            umma_f16(tmem + 192, imh, cl, idesc, first);   // D2 im
            umma_f16(tmem + 192, iml, ch, idesc, 1);
            umma_f16(tmem + 192, reh, nl, idesc, 1);
            umma_f16(tmem + 192, rel, nh, idesc, 1);
        }
    }
}

// Largest value over the block (N1 = 64: the two threads of a row and the
// lines of a tile share one scale); `red` holds THREADS / 32 floats.
template <int N1>
__device__ __forceinline__ float t5_block_max(float m, float *red) {
#pragma unroll
    for (int off = 16; off > 0; off >>= 1) m = fmaxf(m, __shfl_xor_sync(0xffffffffu, m, off));
    if ((threadIdx.x & 31) == 0) red[threadIdx.x >> 5] = m;
    __syncthreads();
    float r = 0.f;
#pragma unroll
    for (int w = 0; w < T5<N1>::THREADS / 32; w++) r = fmaxf(r, red[w]);
    __syncthreads();  // red is reused by the next reduction
    return r;
}

// Lines of a launch: every row (ROWS) or every column of `images` images;
// the line length (cols resp. rows) is N1^2 and the line count a multiple of
// 128 / N1.
template <int N1, bool ROWS>
__global__ void __launch_bounds__(T5<N1>::THREADS, T5<N1>::BLOCKS)
    tc5_lines(const PassArgs a, const uint4 *__restrict__ g_dft, const float2 *__restrict__ g_tw,
              int images) {
    using S = T5<N1>;
    constexpr int N = S::N;
    extern __shared__ __align__(1024) unsigned char t5_raw[];
    // the swizzle follows absolute shared-memory address bits: the operands
    // need a 1024-byte aligned base (the dynamic shared memory of a kernel
    // without static shared memory starts there; checked, never assumed)
    if (smem_u32(t5_raw) & 1023u) {
        if (threadIdx.x == 0 && a.err) atomicExch(a.err, (int)GLSFFT_ERROR_MISALIGNED);
        return;
    }
    unsigned char *base = t5_raw;
    unsigned char *op_hi = base;
    unsigned char *op_lo = base + S::OP;
    unsigned char *dft_hi = base + 2 * S::OP;
    unsigned char *dft_lo = dft_hi + S::DFT;
    unsigned long long *bar = reinterpret_cast<unsigned long long *>(dft_lo + S::DFT);
    unsigned *tslot = reinterpret_cast<unsigned *>(bar + 1);
    float *red = reinterpret_cast<float *>(bar + 8);

    const int tid = threadIdx.x, lane = tid & 31;
    const int row = tid & 127;              // GEMM row (TMEM lane)
    const int half = tid >> 7;              // N1 = 64: which 32 values of the row
    const int q = (tid >> 5) & 3;           // TMEM lane quarter of this warp
    const int l_in_tile = row / N1, pos = row % N1;  // (line, n2) resp. (line, k1)
    // the DFT matrix, hi then lo, already in the swizzled operand layout
    for (int i = tid; i < (int)(2 * S::DFT / 16); i += S::THREADS)
        reinterpret_cast<uint4 *>(dft_hi)[i] = __ldg(g_dft + i);
    if (tid == 0) {
        mbar_init(bar, 1);
        asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
    }
    if (tid < 32) tmem_alloc<S::TCOLS>(tslot);
    pdl_enter();
    fence_async_smem();
    tc_fence_before();
    __syncthreads();
    tc_fence_after();
    const unsigned tmem = *tslot;
    const unsigned trow = tmem + ((unsigned)(q * 32) << 16) + (unsigned)(32 * half);
    const unsigned s_hi = smem_u32(op_hi), s_lo = smem_u32(op_lo);
    const unsigned s_dh = smem_u32(dft_hi), s_dl = smem_u32(dft_lo);

    const int lines = ROWS ? a.rows : a.cols;
    const int tpi = lines / S::LINES;
    const int total = tpi * images;
    const bool cin = a.flags & PF_CONJ_IN;
    const float osc = a.scale, osi = (a.flags & PF_CONJ_OUT) ? -a.scale : a.scale;
    const bool shift = a.flags & (ROWS ? PF_SHIFT_COLS : PF_SHIFT_ROWS);
    unsigned phase = 0;
    bool failed = false;

    for (int tile = blockIdx.x; tile < total; tile += gridDim.x) {
        const int img = tile / tpi;
        const int line = (tile % tpi) * S::LINES + l_in_tile;
        const float2 *in = static_cast<const float2 *>(image_in(a, img));
        float2 *out = static_cast<float2 *>(image_out(a, img));

        // ---- stage A operand: row (line, n2 = pos), n1 = 32 half + i
        float2 v[32];
#pragma unroll
        for (int i = 0; i < 32; i++) {
            const int n = N1 * (32 * half + i) + pos;
            v[i] = ROWS ? __ldg(in + (size_t)line * N + n) : __ldg(in + (size_t)n * a.cols + line);
        }
        float m = 0.f;
#pragma unroll
        for (int i = 0; i < 32; i++) {
            if (cin) v[i].y = -v[i].y;
            m = fmaxf(m, fmaxf(fabsf(v[i].x), fabsf(v[i].y)));
        }
        const float sa = pow2_scale(N1 == 32 ? m : t5_block_max<N1>(m, red));
#pragma unroll
        for (int j = 0; j < 8; j++) {  // chunk j: re (j < 4) or im of n1 = 32 half + 8 (j % 4) ..
            __half h[8], l[8];
#pragma unroll
            for (int e = 0; e < 8; e++) {
                const float2 z = v[(j & 3) * 8 + e];
                split_half((j < 4 ? z.x : z.y) * sa, h[e], l[e]);
            }
            const unsigned k = (unsigned)((j < 4 ? 0 : N1) + 32 * half + 8 * (j & 3));
            const unsigned off = op_offset((unsigned)row, k);
            *reinterpret_cast<uint4 *>(op_hi + off) = pack8(h);
            *reinterpret_cast<uint4 *>(op_lo + off) = pack8(l);
        }
        fence_async_smem();
        tc_fence_before();
        __syncthreads();
        if (tid == 0) {
            tc_fence_after();
            t5_products<N1>(s_hi, s_lo, s_dh, s_dl, tmem);
            umma_commit(bar);
        }
        bool ok = mbar_wait(bar, phase, kT5WaitNs);
        phase ^= 1u;
        if (__syncthreads_or(!ok)) {
            failed = true;
            break;
        }
        tc_fence_after();

        // ---- stage B on row (line, n2 = pos): Y'[k1], k1 = 32 half + i
        const float ia = 1.0f / sa;  // exact: a power of two
        float yr[32], yi[32];
#pragma unroll
        for (int c = 0; c < 4; c++) {
            float d[32];  // D1 re, D1 im, D2 re, D2 im
            tmem_ld_4x8(trow + 8 * c, trow + N1 + 8 * c, trow + 2 * N1 + 8 * c,
                        trow + 3 * N1 + 8 * c, d);
#pragma unroll
            for (int e = 0; e < 8; e++) {
                const int i = 8 * c + e, k1 = 32 * half + i;
                const float2 y = make_float2((d[e] + d[16 + e]) * ia, (d[8 + e] + d[24 + e]) * ia);
                const float2 w = __ldg(g_tw + k1 * N1 + pos);
                const float2 z = cmul(y, w);
                yr[i] = z.x;
                yi[i] = z.y;
            }
        }
        // ---- stage C operand: rows (line, k1), K = (re, im) of n2 = pos;
        // N1 = 32: one power-of-two scale per line (this warp), N1 = 64: per tile
        float mc = 0.f;
#pragma unroll
        for (int i = 0; i < 32; i++) mc = fmaxf(mc, fmaxf(fabsf(yr[i]), fabsf(yi[i])));
        if constexpr (N1 == 32) {
#pragma unroll
            for (int off = 16; off > 0; off >>= 1) mc = fmaxf(mc, __shfl_xor_sync(0xffffffffu, mc, off));
        } else {
            mc = t5_block_max<N1>(mc, red);
        }
        const float sc = pow2_scale(mc);
#pragma unroll
        for (int i = 0; i < 32; i++) {
            const unsigned rr = (unsigned)(l_in_tile * N1 + 32 * half + i);
            __half hr, lr, hm, lm;
            split_half(yr[i] * sc, hr, lr);
            split_half(yi[i] * sc, hm, lm);
            const unsigned ore = op_offset(rr, (unsigned)pos);
            const unsigned oim = op_offset(rr, (unsigned)(N1 + pos));
            *reinterpret_cast<__half *>(op_hi + ore) = hr;
            *reinterpret_cast<__half *>(op_lo + ore) = lr;
            *reinterpret_cast<__half *>(op_hi + oim) = hm;
            *reinterpret_cast<__half *>(op_lo + oim) = lm;
        }
        fence_async_smem();
        tc_fence_before();  // this thread's accumulator reads are complete
        __syncthreads();
        if (tid == 0) {
            tc_fence_after();
            t5_products<N1>(s_hi, s_lo, s_dh, s_dl, tmem);
            umma_commit(bar);
        }
        ok = mbar_wait(bar, phase, kT5WaitNs);
        phase ^= 1u;
        if (__syncthreads_or(!ok)) {
            failed = true;
            break;
        }
        tc_fence_after();

        // ---- output: row (line, k1 = pos) holds out[k1 + N1 k2], k2 = 32 half + i
        const float icr = osc / sc, ici = osi / sc;
#pragma unroll
        for (int c = 0; c < 4; c++) {
            float d[32];
            tmem_ld_4x8(trow + 8 * c, trow + N1 + 8 * c, trow + 2 * N1 + 8 * c,
                        trow + 3 * N1 + 8 * c, d);
#pragma unroll
            for (int e = 0; e < 8; e++) {
                const int k2 = 32 * half + 8 * c + e;
                const float2 o = make_float2((d[e] + d[16 + e]) * icr, (d[8 + e] + d[24 + e]) * ici);
                int p = pos + N1 * k2;
                if (shift) p = (p + N / 2) & (N - 1);
                if (ROWS) out[(size_t)line * N + p] = o;
                else out[(size_t)p * a.cols + line] = o;
            }
        }
        tc_fence_before();  // before the next tile's products overwrite the accumulators
    }
    if (failed && tid == 0 && a.err) atomicExch(a.err, (int)GLSFFT_ERROR_TIMEOUT);
    tc_fence_before();
    __syncthreads();
    if (tid < 32) tmem_dealloc<S::TCOLS>(tmem);
}

template <int N1, bool ROWS>
cudaError_t t5_launch(const PassArgs &a, const TcTables &t, int images, cudaStream_t s) {
    using S = T5<N1>;
    auto kern = tc5_lines<N1, ROWS>;
    cudaError_t e = smem_opt_in(reinterpret_cast<const void *>(kern), S::SMEM);
    if (e != cudaSuccess) return e;
    int dev = 0, sms = 0;
    e = cudaGetDevice(&dev);
    if (e == cudaSuccess) e = cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
    if (e != cudaSuccess) return e;
    const int lines = ROWS ? a.rows : a.cols;
    const long long total = (long long)(lines / S::LINES) * images;
    const long long cap = (long long)sms * S::BLOCKS;
    const int grid = (int)(total < cap ? total : cap);
    if (grid < 1) return cudaSuccess;
    const uint4 *dft = reinterpret_cast<const uint4 *>(N1 == 32 ? t.dft32_sw : t.dft64_sw);
    const float2 *tw = N1 == 32 ? t.tw1024 : t.tw4096;
    return launch_maybe_pdl(a.pdl != 0, kern, dim3(grid), dim3(S::THREADS), S::SMEM, s, a, dft, tw,
                            images);
}

}  // namespace

cudaError_t launch_tc5_lines(int n, bool rows, const PassArgs &a, const TcTables &t, int images,
                             cudaStream_t s) {
    if (n == 1024) return rows ? t5_launch<32, true>(a, t, images, s) : t5_launch<32, false>(a, t, images, s);
    if (n == 4096) return rows ? t5_launch<64, true>(a, t, images, s) : t5_launch<64, false>(a, t, images, s);
    return cudaErrorInvalidValue;
}

// The real form of the N1-point DFT as B operand images (K-major, 128-byte
// swizzle), FP16 hi then lo.  cos_sin[m] = {cos, sin}(2 pi m / N1).
// N1 = 32: one 64 x 64 matrix, row (c, k1), column (c', n1):
//   [re out] = [ C  S] [re in]     [im out] = [-S  C] [re in; im in]
// N1 = 64: three 64 x 64 blocks C, S, -S, row k1, column n1.
void tc5_dft_image(int n1, const double (*cos_sin)[2], unsigned char *dst) {
    const unsigned blk = 64 * 128;
    const unsigned split = n1 == 32 ? blk : 3 * blk;  // bytes of one split
    for (unsigned i = 0; i < 2 * split; i++) dst[i] = 0;
    auto put = [&](unsigned block, int row, int k, double v) {
        const __half h = __double2half(v);
        const __half l = __double2half(v - (double)__half2float(h));
        const unsigned off = block * blk + sw128_offset((unsigned)row, (unsigned)k);
        *reinterpret_cast<__half *>(dst + off) = h;
        *reinterpret_cast<__half *>(dst + split + off) = l;
    };
    if (n1 == 32) {
        for (int row = 0; row < 64; row++)
            for (int k = 0; k < 64; k++) {
                const int c = row / 32, k1 = row % 32, cp = k / 32, nn = k % 32;
                const double cs = cos_sin[(nn * k1) % 32][0], sn = cos_sin[(nn * k1) % 32][1];
                put(0, row, k, c == 0 ? (cp == 0 ? cs : sn) : (cp == 0 ? -sn : cs));
            }
    } else {
        for (int k1 = 0; k1 < 64; k1++)
            for (int nn = 0; nn < 64; nn++) {
                const double cs = cos_sin[(nn * k1) % 64][0], sn = cos_sin[(nn * k1) % 64][1];
                put(0, k1, nn, cs);
                put(1, k1, nn, sn);
                put(2, k1, nn, -sn);
            }
    }
}

}  // namespace glsfft
