// fft_cols.cu -- instantiations and launcher of the column-pass kernel.
#include "fft_config.h"
#include "fft_kernels.cuh"

namespace glsfft {

template <int N, int LD, int ST>
static cudaError_t cols_t(const PassArgs &a, int images, cudaStream_t s) {
    constexpr int E = cols_E(N), W = cols_W(N), T = cols_T(N);
    constexpr int threads = W * T;
    constexpr size_t smem = num_passes(N) > 1 ? sizeof(float2) * (size_t)padded_count(N * W) : 0;
    auto kern = fft_cols_kernel<N, E, W, LD, ST>;
    if constexpr (smem > 48 * 1024) {
        const cudaError_t e = smem_opt_in(reinterpret_cast<const void *>(kern), smem);
        if (e != cudaSuccess) return e;
    }
    dim3 grid((a.cols + W - 1) / W, images);
    return launch_pass(kern, grid, threads, smem, s, a);
}

template <int LD, int ST>
static cudaError_t cols_n(int n, const PassArgs &a, int images, cudaStream_t s) {
    switch (n) {
    case 1: return cols_t<1, LD, ST>(a, images, s);
    case 2: return cols_t<2, LD, ST>(a, images, s);
    case 4: return cols_t<4, LD, ST>(a, images, s);
    case 8: return cols_t<8, LD, ST>(a, images, s);
    case 16: return cols_t<16, LD, ST>(a, images, s);
    case 32: return cols_t<32, LD, ST>(a, images, s);
    case 64: return cols_t<64, LD, ST>(a, images, s);
    case 128: return cols_t<128, LD, ST>(a, images, s);
    case 256: return cols_t<256, LD, ST>(a, images, s);
    case 512: return cols_t<512, LD, ST>(a, images, s);
    case 1024: return cols_t<1024, LD, ST>(a, images, s);
    case 2048: return cols_t<2048, LD, ST>(a, images, s);
    case 4096: return cols_t<4096, LD, ST>(a, images, s);
    default: return cudaErrorInvalidValue;
    }
}

cudaError_t launch_cols(int n, int ld, int st, const PassArgs &a, int images, cudaStream_t s) {
    if (ld == LD_C2 && st == ST_C2) return cols_n<LD_C2, ST_C2>(n, a, images, s);
    if (ld == LD_C2 && st == ST_LOGMAG_MINMAX) return cols_n<LD_C2, ST_LOGMAG_MINMAX>(n, a, images, s);
    return cudaErrorInvalidValue;
}

}  // namespace glsfft
