// tc5_fft.cu -- precision form on the fifth-generation tensor cores: 1024-point
// line FFTs (rows or columns of CV_32FC2 images) as a 32 x 32 four-step whose
// two DFT stages are tcgen05 matrix products with FP16 hi/lo split operands
// (hi*hi into one FP32 accumulator, hi*lo + lo*hi into a second, both in
// tensor memory), so the result keeps FP32-level error.
//
// A line x of N = 1024 points is the 32 x 32 matrix X[n1][n2] = x[32 n1 + n2]:
//   stage A  Y[k1][n2] = sum_n1 x[32 n1 + n2] e^{-2 pi i n1 k1 / 32}
//   stage B  Y'[k1][n2] = Y[k1][n2] e^{-2 pi i k1 n2 / 1024}
//   stage C  out[k1 + 32 k2] = sum_n2 Y'[k1][n2] e^{-2 pi i n2 k2 / 32}
// Both DFT stages are one GEMM over a tile of 4 lines: 128 rows (line, n2)
// resp. (line, k1), K = 64 (real parts then imaginary parts of the 32 inputs),
// N = 64 (real then imaginary parts of the 32 outputs) against the real form
// of the 32-point DFT matrix.  Each thread owns one GEMM row: it loads its 32
// inputs, splits them after a power-of-two row scale (hi = fp16(v), lo =
// fp16(v - hi)) into the A operands in shared memory, and reads its row of
// the accumulators back from tensor memory.  Stage B and the stage-C operand
// build (a transposing write, conflict-free in the 128-byte-swizzled layout)
// happen between the two products; stage C's operand is scaled per line.
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

constexpr int kT5Threads = 128;             // one thread per GEMM row
constexpr int kT5Lines = 4;                 // 1024-point lines per tile
constexpr unsigned kT5OpBytes = 128 * 128;  // a 128-row x 64-half operand
constexpr unsigned kT5DftBytes = 64 * 128;  // the 64 x 64-half DFT matrix
constexpr size_t kT5Smem = 2 * kT5OpBytes + 2 * kT5DftBytes + 64 + 1024;  // + alignment slack
constexpr long long kT5WaitNs = 2000000000ll;
constexpr int kT5BlocksPerSm = 4;           // 4 x 128 TMEM columns = all 512

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

// The three products of one DFT stage, K = 64 in four steps of 16:
// D1 (TMEM columns 0-63) = Ahi Bhi, D2 (columns 64-127) = Ahi Blo + Alo Bhi.
__device__ __forceinline__ void t5_products(unsigned a_hi, unsigned a_lo, unsigned b_hi,
                                            unsigned b_lo, unsigned tmem) {
    constexpr uint32_t idesc = umma_idesc_f16(128, 64);
#pragma unroll
    for (int kk = 0; kk < 4; kk++) {
        const uint64_t ah = umma_desc_sw128(a_hi + 32 * kk), al = umma_desc_sw128(a_lo + 32 * kk);
        const uint64_t bh = umma_desc_sw128(b_hi + 32 * kk), bl = umma_desc_sw128(b_lo + 32 * kk);
        umma_f16(tmem, ah, bh, idesc, kk > 0);
        umma_f16(tmem + 64, ah, bl, idesc, kk > 0);
        umma_f16(tmem + 64, al, bh, idesc, 1);
    }
}

// Lines of a launch: every row (ROWS) or every column of `images` images;
// the line length (cols resp. rows) is 1024 and the line count a multiple of 4.
template <bool ROWS>
__global__ void __launch_bounds__(kT5Threads, kT5BlocksPerSm)
    tc5_lines_1024(const PassArgs a, const uint4 *__restrict__ g_dft,
                   const float2 *__restrict__ g_tw, int images) {
    extern __shared__ __align__(1024) unsigned char t5_raw[];
    // the swizzle follows absolute shared-memory address bits: 1024-byte base
    unsigned char *base = t5_raw + ((1024u - (smem_u32(t5_raw) & 1023u)) & 1023u);
    unsigned char *op_hi = base;
    unsigned char *op_lo = base + kT5OpBytes;
    unsigned char *dft_hi = base + 2 * kT5OpBytes;
    unsigned char *dft_lo = dft_hi + kT5DftBytes;
    unsigned long long *bar = reinterpret_cast<unsigned long long *>(dft_lo + kT5DftBytes);
    unsigned *tslot = reinterpret_cast<unsigned *>(bar + 1);

    const int tid = threadIdx.x, warp = tid >> 5, lane = tid & 31;
    // the DFT matrix, hi then lo, already in the swizzled operand layout
    for (int i = tid; i < (int)(2 * kT5DftBytes / 16); i += kT5Threads)
        reinterpret_cast<uint4 *>(dft_hi)[i] = __ldg(g_dft + i);
    if (tid == 0) {
        mbar_init(bar, 1);
        asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
    }
    if (warp == 0) tmem_alloc<128>(tslot);
    pdl_enter();
    fence_async_smem();
    tc_fence_before();
    __syncthreads();
    tc_fence_after();
    const unsigned tmem = *tslot;
    const unsigned trow = tmem + ((unsigned)(warp * 32) << 16);  // this warp's TMEM lanes
    const unsigned s_hi = smem_u32(op_hi), s_lo = smem_u32(op_lo);
    const unsigned s_dh = smem_u32(dft_hi), s_dl = smem_u32(dft_lo);

    const int lines = ROWS ? a.rows : a.cols;
    const int tpi = lines / kT5Lines;
    const int total = tpi * images;
    const bool cin = a.flags & PF_CONJ_IN;
    const float osc = a.scale, osi = (a.flags & PF_CONJ_OUT) ? -a.scale : a.scale;
    const bool shift = a.flags & (ROWS ? PF_SHIFT_COLS : PF_SHIFT_ROWS);
    unsigned phase = 0;
    bool failed = false;

    for (int tile = blockIdx.x; tile < total; tile += gridDim.x) {
        const int img = tile / tpi;
        const int line = (tile % tpi) * kT5Lines + warp;
        const float2 *in = static_cast<const float2 *>(image_in(a, img));
        float2 *out = static_cast<float2 *>(image_out(a, img));

        // ---- stage A operand: row (line, n2 = lane), K = (re, im) of n1 = 0..31
        float2 v[32];
#pragma unroll
        for (int n1 = 0; n1 < 32; n1++)
            v[n1] = ROWS ? __ldg(in + (size_t)line * 1024 + 32 * n1 + lane)
                         : __ldg(in + (size_t)(32 * n1 + lane) * a.cols + line);
        float m = 0.f;
#pragma unroll
        for (int n1 = 0; n1 < 32; n1++) {
            if (cin) v[n1].y = -v[n1].y;
            m = fmaxf(m, fmaxf(fabsf(v[n1].x), fabsf(v[n1].y)));
        }
        const float sa = pow2_scale(m);
#pragma unroll
        for (int j = 0; j < 8; j++) {  // 16-byte chunk j: re (j < 4) or im of n1 = 8(j%4) ..
            __half h[8], l[8];
#pragma unroll
            for (int e = 0; e < 8; e++) {
                const float2 q = v[(j & 3) * 8 + e];
                split_half((j < 4 ? q.x : q.y) * sa, h[e], l[e]);
            }
            const unsigned off = (unsigned)(tid >> 3) * 1024 + (unsigned)(tid & 7) * 128 +
                                 ((unsigned)(j ^ (tid & 7)) << 4);
            *reinterpret_cast<uint4 *>(op_hi + off) = pack8(h);
            *reinterpret_cast<uint4 *>(op_lo + off) = pack8(l);
        }
        fence_async_smem();
        tc_fence_before();
        __syncthreads();
        if (tid == 0) {
            tc_fence_after();
            t5_products(s_hi, s_lo, s_dh, s_dl, tmem);
            umma_commit(bar);
        }
        bool ok = mbar_wait(bar, phase, kT5WaitNs);
        phase ^= 1u;
        if (__syncthreads_or(!ok)) {
            failed = true;
            break;
        }
        tc_fence_after();

        // ---- stage B on this thread's row (line, n2 = lane): Y'[k1]
        const float ia = 1.0f / sa;  // exact: a power of two
        float yr[32], yi[32];
#pragma unroll
        for (int c = 0; c < 4; c++) {  // k1 = 8c .. 8c + 7
            float d[32];  // D1 re, D1 im, D2 re, D2 im
            tmem_ld_4x8(trow + 8 * c, trow + 32 + 8 * c, trow + 64 + 8 * c, trow + 96 + 8 * c, d);
#pragma unroll
            for (int e = 0; e < 8; e++) {
                const int k1 = 8 * c + e;
                const float2 y = make_float2((d[e] + d[16 + e]) * ia, (d[8 + e] + d[24 + e]) * ia);
                const float2 w = __ldg(g_tw + k1 * 32 + lane);
                const float2 z = cmul(y, w);
                yr[k1] = z.x;
                yi[k1] = z.y;
            }
        }
        // ---- stage C operand: rows (line, k1), K = (re, im) of n2 = lane;
        // one power-of-two scale per line (this warp)
        float mc = 0.f;
#pragma unroll
        for (int k1 = 0; k1 < 32; k1++) mc = fmaxf(mc, fmaxf(fabsf(yr[k1]), fabsf(yi[k1])));
#pragma unroll
        for (int off = 16; off > 0; off >>= 1) mc = fmaxf(mc, __shfl_xor_sync(0xffffffffu, mc, off));
        const float sc = pow2_scale(mc);
#pragma unroll
        for (int k1 = 0; k1 < 32; k1++) {
            const unsigned rr = (unsigned)(warp * 32 + k1);
            __half hr, lr, hm, lm;
            split_half(yr[k1] * sc, hr, lr);
            split_half(yi[k1] * sc, hm, lm);
            const unsigned ore = sw128_offset(rr, (unsigned)lane);
            const unsigned oim = sw128_offset(rr, 32u + (unsigned)lane);
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
            t5_products(s_hi, s_lo, s_dh, s_dl, tmem);
            umma_commit(bar);
        }
        ok = mbar_wait(bar, phase, kT5WaitNs);
        phase ^= 1u;
        if (__syncthreads_or(!ok)) {
            failed = true;
            break;
        }
        tc_fence_after();

        // ---- output: row (line, k1 = lane) holds out[k1 + 32 k2], k2 = 0..31
        const float icr = osc / sc, ici = osi / sc;
#pragma unroll
        for (int c = 0; c < 4; c++) {
            float d[32];
            tmem_ld_4x8(trow + 8 * c, trow + 32 + 8 * c, trow + 64 + 8 * c, trow + 96 + 8 * c, d);
#pragma unroll
            for (int e = 0; e < 8; e++) {
                const int k2 = 8 * c + e;
                const float2 o = make_float2((d[e] + d[16 + e]) * icr, (d[8 + e] + d[24 + e]) * ici);
                int p = lane + 32 * k2;
                if (shift) p = (p + 512) & 1023;
                if (ROWS) out[(size_t)line * 1024 + p] = o;
                else out[(size_t)p * a.cols + line] = o;
            }
        }
        tc_fence_before();  // before the next tile's products overwrite the accumulators
    }
    if (failed && tid == 0 && a.err) atomicExch(a.err, (int)GLSFFT_ERROR_TIMEOUT);
    tc_fence_before();
    __syncthreads();
    if (warp == 0) tmem_dealloc<128>(tmem);
}

template <bool ROWS>
cudaError_t t5_launch(const PassArgs &a, const TcTables &t, int images, cudaStream_t s) {
    auto kern = tc5_lines_1024<ROWS>;
    cudaError_t e = smem_opt_in(reinterpret_cast<const void *>(kern), kT5Smem);
    if (e != cudaSuccess) return e;
    int dev = 0, sms = 0;
    e = cudaGetDevice(&dev);
    if (e == cudaSuccess) e = cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
    if (e != cudaSuccess) return e;
    const int lines = ROWS ? a.rows : a.cols;
    const long long total = (long long)(lines / kT5Lines) * images;
    const long long cap = (long long)sms * kT5BlocksPerSm;
    const int grid = (int)(total < cap ? total : cap);
    if (grid < 1) return cudaSuccess;
    return launch_maybe_pdl(a.pdl != 0, kern, dim3(grid), dim3(kT5Threads), kT5Smem, s, a,
                            reinterpret_cast<const uint4 *>(t.dft32_sw), t.tw1024, images);
}

}  // namespace

cudaError_t launch_tc5_lines_1024(bool rows, const PassArgs &a, const TcTables &t, int images,
                                  cudaStream_t s) {
    return rows ? t5_launch<true>(a, t, images, s) : t5_launch<false>(a, t, images, s);
}

// The real form of the 32-point DFT as the B operand (64 x 64, K-major):
// row (c, k1), column (c', n1) with cos, sin of 2 pi n1 k1 / 32:
//   [re out] = [ cos  sin] [re in]      [im out] = [-sin  cos] [re in; im in]
// split into FP16 hi/lo and laid out as the 128-byte-swizzled operand image.
void tc5_dft32_image(const double (*cos_sin)[2], unsigned char *dst16k) {
    for (int i = 0; i < (int)(2 * kT5DftBytes); i++) dst16k[i] = 0;
    for (int row = 0; row < 64; row++)
        for (int k = 0; k < 64; k++) {
            const int c = row / 32, k1 = row % 32, cp = k / 32, n1 = k % 32;
            const double cs = cos_sin[(n1 * k1) % 32][0], sn = cos_sin[(n1 * k1) % 32][1];
            const double v = c == 0 ? (cp == 0 ? cs : sn) : (cp == 0 ? -sn : cs);
            const __half h = __double2half(v);
            const __half l = __double2half(v - (double)__half2float(h));
            const unsigned off = sw128_offset((unsigned)row, (unsigned)k);
            *reinterpret_cast<__half *>(dst16k + off) = h;
            *reinterpret_cast<__half *>(dst16k + kT5DftBytes + off) = l;
        }
}

}  // namespace glsfft
