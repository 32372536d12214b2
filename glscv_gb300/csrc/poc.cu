// poc.cu -- fused phaseCorrelate column kernel (the centroid finish is fused
// into the inverse row pass, fft_kernels.cuh).
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
        const cudaError_t e = smem_opt_in(reinterpret_cast<const void *>(kern), smem);
        if (e != cudaSuccess) return e;
    }
    dim3 grid((a.cols + W - 1) / W, 1);
    return launch_pass(kern, grid, threads, smem, s, a);
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

}  // namespace glsfft
