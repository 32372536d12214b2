// fft_rows.cu -- instantiations and launcher of the row-pass kernel.
#include "fft_config.h"
#include "fft_kernels.cuh"

namespace glsfft {

// The real-input and argmax row passes (phaseCorrelate, the FFT display,
// promoted CV_32FC1 input) take row schedule 2's shape on 2048- and
// 4096-point rows -- 32 values per thread, as the complex pass does by
// default there -- with the same radix order, so the same results.
template <int N, int LD, int ST>
constexpr PassShape rows_fixed_shape() {
    return (N >= 2048 && !(LD == LD_C2 && ST == ST_C2)) ? row_shape(N, 2) : row_shape(N, 0);
}

template <int N, int LD, int ST>
static cudaError_t rows_t(const PassArgs &a, int images, cudaStream_t s) {
    constexpr PassShape sh = rows_fixed_shape<N, LD, ST>();
    constexpr int E = sh.E, LINES = sh.G, T = N / E;
    constexpr int threads = LINES * T;
    constexpr size_t smem = num_passes(N) > 1 ? sizeof(float2) * (size_t)LINES * padded_count(N) : 0;
    auto kern = fft_rows_kernel<N, E, LINES, LD, ST, sh.MB>;
    if constexpr (smem > 48 * 1024) {
        const cudaError_t e = smem_opt_in(reinterpret_cast<const void *>(kern), smem);
        if (e != cudaSuccess) return e;
    }
    dim3 grid((a.rows + LINES - 1) / LINES, images);
    return launch_pass(kern, grid, threads, smem, s, a);
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
