// fft_rows.cu -- instantiations and launcher of the row-pass kernel.
#include "fft_config.h"
#include "fft_kernels.cuh"

namespace glsfft {

template <int N, int LD, int ST>
static cudaError_t rows_t(const PassArgs &a, int images, cudaStream_t s) {
    constexpr int E = rows_E(N), LINES = rows_LINES(N), T = rows_T(N);
    constexpr int threads = LINES * T;
    constexpr size_t smem = num_passes(N) > 1 ? sizeof(float2) * (size_t)LINES * padded_count(N) : 0;
    auto kern = fft_rows_kernel<N, E, LINES, LD, ST>;
    if constexpr (smem > 48 * 1024) {
        const cudaError_t e = smem_opt_in(reinterpret_cast<const void *>(kern), smem);
        if (e != cudaSuccess) return e;
    }
    dim3 grid((a.rows + LINES - 1) / LINES, images);
    kern<<<grid, threads, smem, s>>>(a);
    return cudaGetLastError();
}

template <int LD, int ST>
static cudaError_t rows_n(int n, const PassArgs &a, int images, cudaStream_t s) {
    switch (n) {
    case 1: return rows_t<1, LD, ST>(a, images, s);
    case 2: return rows_t<2, LD, ST>(a, images, s);
    case 4: return rows_t<4, LD, ST>(a, images, s);
    case 8: return rows_t<8, LD, ST>(a, images, s);
    case 16: return rows_t<16, LD, ST>(a, images, s);
    case 32: return rows_t<32, LD, ST>(a, images, s);
    case 64: return rows_t<64, LD, ST>(a, images, s);
    case 128: return rows_t<128, LD, ST>(a, images, s);
    case 256: return rows_t<256, LD, ST>(a, images, s);
    case 512: return rows_t<512, LD, ST>(a, images, s);
    case 1024: return rows_t<1024, LD, ST>(a, images, s);
    case 2048: return rows_t<2048, LD, ST>(a, images, s);
    case 4096: return rows_t<4096, LD, ST>(a, images, s);
    default: return cudaErrorInvalidValue;
    }
}

cudaError_t launch_rows(int n, int ld, int st, const PassArgs &a, int images, cudaStream_t s) {
    if (ld == LD_C2 && st == ST_C2) return rows_n<LD_C2, ST_C2>(n, a, images, s);
    if (ld == LD_R1 && st == ST_C2) return rows_n<LD_R1, ST_C2>(n, a, images, s);
    if (ld == LD_R1W && st == ST_C2) return rows_n<LD_R1W, ST_C2>(n, a, images, s);
    if (ld == LD_C2 && st == ST_RE_ARGMAX) return rows_n<LD_C2, ST_RE_ARGMAX>(n, a, images, s);
    return cudaErrorInvalidValue;
}

}  // namespace glsfft
