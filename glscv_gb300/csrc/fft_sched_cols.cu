// fft_sched_cols.cu -- schedules 1..kPassSchedules-1 of the complex column pass
// (fft_config.h), for the autotuner; schedule 0 is fft_cols.cu's.
#include "fft_config.h"
#include "fft_kernels.cuh"
#include "sched_internal.h"

namespace glsfft {

template <int N, int ID>
static cudaError_t cols_s(const PassArgs &a, int images, cudaStream_t s) {
    if constexpr (!sched_available(N, ID, true) || ID == 0) {
        return cudaErrorInvalidValue;
    } else {
        constexpr PassShape sh = col_shape(N, ID);
        constexpr int threads = shape_threads(N, sh);
        constexpr size_t smem = (size_t)shape_smem(N, sh, true);
        auto kern = fft_cols_kernel<N, sh.E, sh.G, LD_C2, ST_C2, sh.MB>;
        if constexpr (smem > 48 * 1024) {
            const cudaError_t e = smem_opt_in(reinterpret_cast<const void *>(kern), smem);
            if (e != cudaSuccess) return e;
        }
        dim3 grid((a.cols + sh.G - 1) / sh.G, images);
        return launch_pass(kern, grid, threads, smem, s, a);
    }
}

template <int ID>
static cudaError_t cols_id(int n, const PassArgs &a, int images, cudaStream_t s) {
    switch (n) {
    case 64: return cols_s<64, ID>(a, images, s);
    case 128: return cols_s<128, ID>(a, images, s);
    case 256: return cols_s<256, ID>(a, images, s);
    case 512: return cols_s<512, ID>(a, images, s);
    case 1024: return cols_s<1024, ID>(a, images, s);
    case 2048: return cols_s<2048, ID>(a, images, s);
    case 4096: return cols_s<4096, ID>(a, images, s);
    default: return cudaErrorInvalidValue;
    }
}

cudaError_t launch_cols_sched(int n, int id, const PassArgs &a, int images, cudaStream_t s) {
    switch (id) {
    case 0: return launch_cols(n, LD_C2, ST_C2, a, images, s);
    case 1: return cols_id<1>(n, a, images, s);
    case 2: return cols_id<2>(n, a, images, s);
    case 3: return cols_id<3>(n, a, images, s);
    case 4: return cols_id<4>(n, a, images, s);
    case 5: return cols_id<5>(n, a, images, s);
    case kSchedStreamed: {
        // arguments the streamed pass does not take run schedule 0
        if (!stream_pass_applies(n, true, a, images)) return launch_cols(n, LD_C2, ST_C2, a, images, s);
        return launch_stream_pass(n, true, a, images, s);
    }
    default: return cudaErrorInvalidValue;
    }
}

}  // namespace glsfft
