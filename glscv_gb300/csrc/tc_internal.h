// tc_internal.h -- tables and launcher of the split-FP16 tensor-core form.
#pragma once
#include <cuda_fp16.h>
#include <cuda_runtime.h>

#include "glsfft_internal.h"

namespace glsfft {

// Device tables, generated in FP64 on the host once per context:
// real-ified DFT matrices [Fr -Fi; Fi Fr] of size 2*N1 split into FP16 hi/lo
// (rows padded to 2*N1 + 8 halves), and the four-step twiddles
// e^{-2 pi i k1 n2 / N} at [k1*N1 + n2].
struct TcTables {
    __half *f32_hi = nullptr, *f32_lo = nullptr;  // N1 = 32 (N = 1024)
    __half *f64_hi = nullptr, *f64_lo = nullptr;  // N1 = 64 (N = 4096)
    float2 *tw1024 = nullptr, *tw4096 = nullptr;
    // the 32-point DFT as the tcgen05 B operand: FP16 hi (8 KB) then lo
    // (8 KB), 128-byte-swizzled K-major image (tc5_fft.cu)
    unsigned char *dft32_sw = nullptr;
    void *block = nullptr;  // one allocation holding all of the above
};

int tc_tables_create(TcTables *t);
void tc_tables_destroy(TcTables *t);

// 1-D FFTs of length n (1024 or 4096) of every row (rows = true) or column.
cudaError_t launch_tc_lines(int n, bool rows, const PassArgs &a, const TcTables &t, int images,
                            cudaStream_t s);

// 1024-point lines on tcgen05 (tc5_fft.cu); the line count must be a
// multiple of 4.
cudaError_t launch_tc5_lines_1024(bool rows, const PassArgs &a, const TcTables &t, int images,
                                  cudaStream_t s);
// Host: the 32-point DFT B operand image (16 KB) from cos_sin[m] =
// {cos, sin}(2 pi m / 32).
void tc5_dft32_image(const double (*cos_sin)[2], unsigned char *dst16k);

}  // namespace glsfft
