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
// A compute thread owns one GEMM row and 32 of its complex values (N1 = 64:
// two threads per row): it reads its inputs from a raw tile staged in shared
// memory, splits them after a power-of-two scale (hi = fp16(v), lo =
// fp16(v - hi)) into the A operands (K-major, 128-byte swizzle), and reads its
// part of the accumulator row back from tensor memory.  Stage B and the
// stage-C operand build (a transposing write, conflict-free in the swizzled
// layout) happen between the products.  A loader warp keeps the next tiles'
// raw inputs in flight (bulk copies for rows, tensor-map boxes for columns)
// while the compute warps work.  One elected thread issues the MMAs;
// completion arrives on mbarriers whose waits are bounded
// (GLSFFT_ERROR_TIMEOUT into the status word on expiry).
//
// Scaling: one power-of-two scale sa per line (or per tile) puts the largest
// input component just under 2^14.  Stage A's accumulator is then sa * Y, so
// sa * Y * w / N1 is bounded by sqrt(2) * 2^14 in every component and goes
// into stage C's operand unscaled; the twiddle table holds w / N1 (exact).
// Stage C's accumulator is (sa / N1) * out, undone by one exact multiply.
#include <cuda_fp16.h>

#include "fft_kernels.cuh"
#include "glsfft.h"
#include "glsfft_internal.h"
#include "tc5_device.cuh"
#include "tc_internal.h"
#include "tma_device.cuh"

namespace glsfft {

namespace {

constexpr long long kT5WaitNs = 2000000000ll;
constexpr unsigned kT5OpBlock = 128 * 128;  // a 128-row x 64-half operand block

// Shapes per N1: compute threads (one per GEMM row and output half), lines
// per tile, A operand bytes (one split), B operand bytes (one split), raw
// input tile bytes and stages, TMEM columns, resident blocks per SM.
template <int N1>
struct T5 {
    static constexpr int N = N1 * N1;
    static constexpr int THREADS = 128 * (N1 / 32);
    static constexpr int LINES = 128 / N1;
    static constexpr unsigned OP = kT5OpBlock * (N1 / 32);         // K = 2 N1 halves
    static constexpr unsigned DFT = N1 == 32 ? 64 * 128 : 3 * 64 * 128;  // [C S;-S C] or C,S,-S
    static constexpr unsigned RAW = (unsigned)LINES * N * 8u;      // one tile, complex FP32
    static constexpr int NST = N1 == 32 ? 2 : 1;
    static constexpr int TCOLS = 4 * N1;                            // D1 re, im; D2 re, im
    static constexpr int BLOCKS = N1 == 32 ? 2 : 1;
    // operands, raw stages, then the mbarriers, TMEM slot, reduction scratch
    // and failure flag; the dynamic shared memory must start 1024-byte
    // aligned (checked in the kernel)
    static constexpr size_t SMEM = 2 * OP + 2 * DFT + (size_t)NST * RAW + 64 + 4 * 64;
};

// power of two putting m just under 2^14 (the FP16 split then keeps 22 bits
// of every value without reaching FP16's range limit in the products)
__device__ __forceinline__ float pow2_scale(float m) {
    if (!(m > 0.f) || !isfinite(m)) return 1.0f;
    int e;
    frexpf(m, &e);  // m = f * 2^e, 0.5 <= f < 1
    return ldexpf(1.0f, 14 - e);
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

// named barrier 1 over the compute warps (the loader warp is not part of it)
__device__ __forceinline__ void bar_compute(int nthreads) {
    asm volatile("bar.sync 1, %0;" ::"r"(nthreads) : "memory");
}
__device__ __forceinline__ bool bar_compute_or(bool pred, int nthreads) {
    unsigned r;
    asm volatile(
        "{\n\t.reg .pred p, q;\n\tsetp.ne.u32 p, %1, 0;\n\t"
        "bar.red.or.pred q, 1, %2, p;\n\tselp.u32 %0, 1, 0, q;\n\t}"
        : "=r"(r)
        : "r"((unsigned)pred), "r"(nthreads)
        : "memory");
    return r != 0;
}

// Largest value over the compute threads (the tile shares one scale); `red`
// holds COMPUTE / 32 floats.
template <int COMPUTE>
__device__ __forceinline__ float t5_tile_max(float m, float *red) {
#pragma unroll
    for (int off = 16; off > 0; off >>= 1) m = fmaxf(m, __shfl_xor_sync(0xffffffffu, m, off));
    if ((threadIdx.x & 31) == 0) red[threadIdx.x >> 5] = m;
    bar_compute(COMPUTE);
    float r = 0.f;
#pragma unroll
    for (int w = 0; w < COMPUTE / 32; w++) r = fmaxf(r, red[w]);
    bar_compute(COMPUTE);  // red is reused by the next reduction
    return r;
}

// One tile's raw input into stage `dst`: a row pass's LINES consecutive rows
// are one contiguous bulk copy; a column pass's LINES adjacent columns arrive
// as 256-row boxes through the tensor map over the whole batch, [row][line].
template <int N1, bool ROWS>
__device__ __forceinline__ void t5_load_tile(const CUtensorMap *tmap, const PassArgs &a, int tile,
                                            int tpi, void *dst, unsigned long long *full) {
    constexpr int N = N1 * N1, LINES = 128 / N1;
    constexpr unsigned BYTES = (unsigned)LINES * N * 8u;
    mbar_arrive_tx(full, BYTES);
    const int img = tile / tpi, line0 = (tile % tpi) * LINES;
    if constexpr (ROWS) {
        const char *src = static_cast<const char *>(a.in0) + (size_t)img * a.in_img_bytes +
                          (size_t)line0 * N * 8u;
        bulk_g2s(dst, src, BYTES, full);
    } else {
#pragma unroll 1
        for (int b = 0; b < N / 256; b++)
            tensor2d_g2s(static_cast<char *>(dst) + (size_t)b * 256 * LINES * 8, tmap, line0,
                         img * a.rows + 256 * b, full);
    }
}

// Lines of a launch: every row (ROWS) or every column of `images` contiguous
// images; the line length (cols resp. rows) is N1^2 and the line count a
// multiple of 128 / N1.  Warps 0 .. COMPUTE/32 - 1 compute; the last warp
// loads tiles ahead into a ring of NST raw stages (a stage is released as
// soon as the compute threads have read their values).
template <int N1, bool ROWS>
__global__ void __launch_bounds__(T5<N1>::THREADS + 32, T5<N1>::BLOCKS)
    tc5_lines(const __grid_constant__ CUtensorMap tmap, const PassArgs a,
              const uint4 *__restrict__ g_dft, const float2 *__restrict__ g_tw, int images) {
    using S = T5<N1>;
    constexpr int N = S::N, COMPUTE = S::THREADS, LINES = S::LINES;
    extern __shared__ __align__(1024) unsigned char t5_raw[];
    // the swizzle follows absolute shared-memory address bits: the operands
    // need a 1024-byte aligned base (the dynamic shared memory of a kernel
    // without static shared memory starts there; checked, never assumed)
    if (smem_u32(t5_raw) & 1023u) {
        if (threadIdx.x == 0 && a.err) atomicExch(a.err, (int)GLSFFT_ERROR_MISALIGNED);
        return;
    }
    unsigned char *op_hi = t5_raw;
    unsigned char *op_lo = t5_raw + S::OP;
    unsigned char *dft_hi = t5_raw + 2 * S::OP;
    unsigned char *dft_lo = dft_hi + S::DFT;
    unsigned char *raw = dft_lo + S::DFT;  // NST stages of RAW bytes
    unsigned long long *full = reinterpret_cast<unsigned long long *>(raw + (size_t)S::NST * S::RAW);
    unsigned long long *empty = full + S::NST;
    unsigned long long *bar = empty + S::NST;  // MMA completion
    unsigned *tslot = reinterpret_cast<unsigned *>(bar + 1);
    float *red = reinterpret_cast<float *>(bar + 2);  // 16 floats
    int &s_failed = *reinterpret_cast<int *>(red + 16);

    const int tid = threadIdx.x, lane = tid & 31;
    const bool loader = tid >= COMPUTE;
    const int row = tid & 127;        // GEMM row (TMEM lane)
    const int half = (tid >> 7) & 1;  // N1 = 64: which 32 values of the row
    const int q = (tid >> 5) & 3;     // TMEM lane quarter of this warp
    // GEMM row <-> (line in the tile, position n2 resp. k1): along a row pass
    // the position runs fastest over the lanes (a warp reads 256 contiguous
    // bytes of one line); along a column pass the line does (a stage holds
    // [row][line], so a warp again reads contiguous bytes, and its stores
    // fill whole 32-byte row segments)
    const int l_in_tile = ROWS ? row / N1 : row % LINES;
    const int pos = ROWS ? row % N1 : row / LINES;
    // the DFT matrix, hi then lo, already in the swizzled operand layout
    for (int i = tid; i < (int)(2 * S::DFT / 16); i += COMPUTE + 32)
        reinterpret_cast<uint4 *>(dft_hi)[i] = __ldg(g_dft + i);
    if (tid == 0) {
        for (int st = 0; st < S::NST; st++) {
            mbar_init(full + st, 1);
            mbar_init(empty + st, COMPUTE);
        }
        mbar_init(bar, 1);
        s_failed = 0;
        asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
    }
    if (tid < 32) tmem_alloc<S::TCOLS>(tslot);
    pdl_enter();
    fence_async_smem();
    tc_fence_before();
    __syncthreads();
    tc_fence_after();
    const unsigned tmem = *tslot;

    const int lines = ROWS ? a.rows : a.cols;
    const int tpi = lines / LINES;
    const int total = tpi * images;

    if (loader) {
        // ---------------------------------------------------------- loader
        if (lane == 0) {
            int it = 0;
            for (int tile = blockIdx.x; tile < total; tile += gridDim.x, it++) {
                const int st = it % S::NST;
                if (it >= S::NST &&
                    !mbar_wait(empty + st, (unsigned)((it / S::NST - 1) & 1), kT5WaitNs)) {
                    s_failed = 1;
                    break;
                }
                t5_load_tile<N1, ROWS>(&tmap, a, tile, tpi, raw + (size_t)st * S::RAW, full + st);
            }
            // no copy may still be writing this block's shared memory when it
            // exits (the compute warps stop early on a failed wait): wait for
            // the last copy issued into each stage (at once if already consumed)
            for (int back = 1; back <= S::NST && back <= it; back++) {
                const int last = it - back;
                mbar_wait(full + last % S::NST, (unsigned)((last / S::NST) & 1), kT5WaitNs);
            }
        }
    } else {
        // --------------------------------------------------------- compute
        const unsigned trow = tmem + ((unsigned)(q * 32) << 16) + (unsigned)(32 * half);
        const unsigned s_hi = smem_u32(op_hi), s_lo = smem_u32(op_lo);
        const unsigned s_dh = smem_u32(dft_hi), s_dl = smem_u32(dft_lo);
        const bool cin = a.flags & PF_CONJ_IN;
        const bool shift = a.flags & (ROWS ? PF_SHIFT_COLS : PF_SHIFT_ROWS);
        // stage C operand: K indices pos (re) and N1 + pos (im) -- their
        // 64-wide block, 16-byte chunk and byte within the chunk; a row adds
        // its atom, its 128-byte line and the chunk swizzle (chunk ^ row % 8)
        const unsigned kre = (unsigned)pos, kim = (unsigned)(N1 + pos);
        const unsigned base_re = (kre >> 6) * kT5OpBlock + (kre & 7) * 2;
        const unsigned base_im = (kim >> 6) * kT5OpBlock + (kim & 7) * 2;
        const unsigned ch_re = (kre & 63) >> 3, ch_im = (kim & 63) >> 3;
        unsigned phase = 0;
        int it = 0;
        for (int tile = blockIdx.x; tile < total; tile += gridDim.x, it++) {
            const int img = tile / tpi;
            const int line = (tile % tpi) * LINES + l_in_tile;
            float2 *out = static_cast<float2 *>(image_out(a, img));
            const int st = it % S::NST;

            // ---- stage A operand: row (line, n2 = pos), n1 = 32 half + i
            bool ok = mbar_wait(full + st, (unsigned)((it / S::NST) & 1), kT5WaitNs);
            if (bar_compute_or(!ok, COMPUTE)) {
                s_failed = 1;
                break;
            }
            const float2 *stage = reinterpret_cast<const float2 *>(raw + (size_t)st * S::RAW);
            float2 v[32];
#pragma unroll
            for (int i = 0; i < 32; i++) {
                const int n1 = 32 * half + i;
                v[i] = ROWS ? stage[l_in_tile * N + N1 * n1 + pos]
                            : stage[(N1 * n1 + pos) * LINES + l_in_tile];
            }
            mbar_arrive(empty + st);  // this thread's part of the stage is read
            float m = 0.f;
#pragma unroll
            for (int i = 0; i < 32; i++) {
                if (cin) v[i].y = -v[i].y;
                m = fmaxf(m, fmaxf(fabsf(v[i].x), fabsf(v[i].y)));
            }
            // one scale per line: a 32-point row pass holds a line per warp,
            // otherwise the tile shares it
            if constexpr (N1 == 32 && ROWS) {
#pragma unroll
                for (int off = 16; off > 0; off >>= 1) m = fmaxf(m, __shfl_xor_sync(0xffffffffu, m, off));
            } else {
                m = t5_tile_max<COMPUTE>(m, red);
            }
            const float sa = pow2_scale(m);
#pragma unroll
            for (int j = 0; j < 8; j++) {  // chunk j: re (j < 4) or im of n1 = 32 half + 8 (j % 4) ..
                unsigned hw[4], lw[4];
#pragma unroll
                for (int e = 0; e < 4; e++) {
                    const float2 z0 = v[(j & 3) * 8 + 2 * e], z1 = v[(j & 3) * 8 + 2 * e + 1];
                    const float x0 = (j < 4 ? z0.x : z0.y) * sa, x1 = (j < 4 ? z1.x : z1.y) * sa;
                    const __half2 h = __floats2half2_rn(x0, x1);
                    const float2 hf = __half22float2(h);
                    const __half2 l = __floats2half2_rn(x0 - hf.x, x1 - hf.y);
                    hw[e] = *reinterpret_cast<const unsigned *>(&h);
                    lw[e] = *reinterpret_cast<const unsigned *>(&l);
                }
                const unsigned k = (unsigned)((j < 4 ? 0 : N1) + 32 * half + 8 * (j & 3));
                const unsigned off = op_offset((unsigned)row, k);
                *reinterpret_cast<uint4 *>(op_hi + off) = make_uint4(hw[0], hw[1], hw[2], hw[3]);
                *reinterpret_cast<uint4 *>(op_lo + off) = make_uint4(lw[0], lw[1], lw[2], lw[3]);
            }
            fence_async_smem();
            tc_fence_before();
            bar_compute(COMPUTE);
            if (tid == 0) {
                tc_fence_after();
                t5_products<N1>(s_hi, s_lo, s_dh, s_dl, tmem);
                umma_commit(bar);
            }
            // stage B's twiddles w^(k1 n2) / N1 for this row, fetched while
            // the products run
            float2 tw[32];
#pragma unroll
            for (int i = 0; i < 32; i++) tw[i] = __ldg(g_tw + (32 * half + i) * N1 + pos);
            ok = mbar_wait(bar, phase, kT5WaitNs);
            phase ^= 1u;
            if (bar_compute_or(!ok, COMPUTE)) {
                s_failed = 1;
                break;
            }
            tc_fence_after();

            // ---- stages B and C operand: row (line, n2 = pos) gives
            // sa Y[k1] w^(k1 n2) / N1 to stage C's rows (line, k1) at K = pos
#pragma unroll
            for (int c = 0; c < 4; c++) {
                float d[32];  // D1 re, D1 im, D2 re, D2 im
                tmem_ld_4x8(trow + 8 * c, trow + N1 + 8 * c, trow + 2 * N1 + 8 * c,
                            trow + 3 * N1 + 8 * c, d);
#pragma unroll
                for (int e = 0; e < 8; e++) {
                    const int i = 8 * c + e, k1 = 32 * half + i;
                    const float2 z = cmul(make_float2(d[e] + d[16 + e], d[8 + e] + d[24 + e]), tw[i]);
                    const __half2 h = __floats2half2_rn(z.x, z.y);
                    const float2 hf = __half22float2(h);
                    const __half2 l = __floats2half2_rn(z.x - hf.x, z.y - hf.y);
                    const unsigned rr = (unsigned)(ROWS ? l_in_tile * N1 + k1 : k1 * LINES + l_in_tile);
                    const unsigned r8 = rr & 7u, rb = (rr >> 3) * 1024u + r8 * 128u;
                    const unsigned ore = base_re + rb + ((ch_re ^ r8) << 4);
                    const unsigned oim = base_im + rb + ((ch_im ^ r8) << 4);
                    *reinterpret_cast<__half *>(op_hi + ore) = __low2half(h);
                    *reinterpret_cast<__half *>(op_lo + ore) = __low2half(l);
                    *reinterpret_cast<__half *>(op_hi + oim) = __high2half(h);
                    *reinterpret_cast<__half *>(op_lo + oim) = __high2half(l);
                }
            }
            fence_async_smem();
            tc_fence_before();  // this thread's accumulator reads are complete
            bar_compute(COMPUTE);
            if (tid == 0) {
                tc_fence_after();
                t5_products<N1>(s_hi, s_lo, s_dh, s_dl, tmem);
                umma_commit(bar);
            }
            ok = mbar_wait(bar, phase, kT5WaitNs);
            phase ^= 1u;
            if (bar_compute_or(!ok, COMPUTE)) {
                s_failed = 1;
                break;
            }
            tc_fence_after();

            // ---- output: row (line, k1 = pos) holds (sa / N1) out[k1 + N1 k2],
            // k2 = 32 half + i; the scale, conjugation and flags' scale in one
            // exact multiply per component
            const float us = (float)N1 / sa;
            const float icr = a.scale * us;
            const float ici = (a.flags & PF_CONJ_OUT) ? -icr : icr;
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
    }
    tc_fence_before();
    __syncthreads();
    if (s_failed && tid == 0 && a.err) atomicExch(a.err, (int)GLSFFT_ERROR_TIMEOUT);
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
    // a column pass reads its tiles through a tensor map over the batch,
    // viewed as one (images * rows) x cols image of 8-byte elements
    CUtensorMap tmap{};
    if (!ROWS &&
        make_tmap_2d(&tmap, a.in0, a.cols, (long long)a.rows * images, S::LINES, 256) != GLSFFT_SUCCESS)
        return cudaErrorNotSupported;
    const uint4 *dft = reinterpret_cast<const uint4 *>(N1 == 32 ? t.dft32_sw : t.dft64_sw);
    const float2 *tw = N1 == 32 ? t.tw1024 : t.tw4096;
    return launch_maybe_pdl(a.pdl != 0, kern, dim3(grid), dim3(S::THREADS + 32), S::SMEM, s, tmap,
                            a, dft, tw, images);
}

}  // namespace

cudaError_t launch_tc_lines(int n, bool rows, const PassArgs &a, const TcTables &t, int images,
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
