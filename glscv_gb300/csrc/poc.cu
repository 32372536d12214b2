// poc.cu -- fused phaseCorrelate column kernel and the centroid finish.
#include "fft_config.h"
#include "fft_kernels.cuh"

namespace glsfft {

template <int N>
static cudaError_t poc_t(const PassArgs &a, cudaStream_t s) {
    constexpr int E = poc_E(N), W = poc_W(N), T = poc_T(N);
    constexpr int threads = W * T;
    constexpr size_t smem = num_passes(N) > 1 ? sizeof(float2) * (size_t)padded_count(N * W) : 0;
    auto kern = poc_cols_kernel<N, E, W>;
    if constexpr (smem > 48 * 1024) {
        static cudaError_t once = cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
        if (once != cudaSuccess) return once;
    }
    dim3 grid((a.cols + W - 1) / W, 1);
    kern<<<grid, threads, smem, s>>>(a);
    return cudaGetLastError();
}

cudaError_t launch_poc_cols(int n, const PassArgs &a, cudaStream_t s) {
    switch (n) {
    case 1: return poc_t<1>(a, s);
    case 2: return poc_t<2>(a, s);
    case 4: return poc_t<4>(a, s);
    case 8: return poc_t<8>(a, s);
    case 16: return poc_t<16>(a, s);
    case 32: return poc_t<32>(a, s);
    case 64: return poc_t<64>(a, s);
    case 128: return poc_t<128>(a, s);
    case 256: return poc_t<256>(a, s);
    case 512: return poc_t<512>(a, s);
    case 1024: return poc_t<1024>(a, s);
    case 2048: return poc_t<2048>(a, s);
    case 4096: return poc_t<4096>(a, s);
    default: return cudaErrorInvalidValue;
    }
}

__global__ void poc_finish_kernel(const float *surface, int rows, int cols, int box,
                                  const unsigned long long *key, double *res) {
    if (blockIdx.x != 0 || threadIdx.x != 0) return;
    const unsigned long long k = *key;
    int px = 0, py = 0;
    double peak = -3.402823466e+38;
    if (k != 0ull) {
        const unsigned idx = key_index(k);
        px = (int)(idx % (unsigned)cols);
        py = (int)(idx / (unsigned)cols);
        peak = (double)key_value(k);
    }
    int minr = py - (box >> 1), maxr = py + (box >> 1);
    int minc = px - (box >> 1), maxc = px + (box >> 1);
    if (minr < 0) minr = 0;
    if (minc < 0) minc = 0;
    if (maxr > rows - 1) maxr = rows - 1;
    if (maxc > cols - 1) maxc = cols - 1;
    double sx = 0.0, sy = 0.0, sum = 0.0;
    for (int y = minr; y <= maxr; y++)
        for (int x = minc; x <= maxc; x++) {
            const double v = (double)surface[(size_t)y * cols + x];
            sx += (double)x * v;
            sy += (double)y * v;
            sum += v;
        }
    const double response = sum / ((double)rows * (double)cols);
    sum += 2.220446049250313e-16;  // DBL_EPSILON, glsPhaseCorrelate.cpp:128
    res[0] = (double)cols / 2.0 - sx / sum;
    res[1] = (double)rows / 2.0 - sy / sum;
    res[2] = response;
    res[3] = (double)(py * cols + px);
    res[4] = peak;
}

cudaError_t launch_poc_finish(const float *surface, int rows, int cols, int box,
                              const unsigned long long *key, double *res, cudaStream_t s) {
    poc_finish_kernel<<<1, 32, 0, s>>>(surface, rows, cols, box, key, res);
    return cudaGetLastError();
}

}  // namespace glsfft
