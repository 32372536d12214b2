// tc_internal.h -- tables and launcher of the split-FP16 tensor-core form.
#pragma once
#include <cuda_fp16.h>
#include <cuda_runtime.h>

#include "glsfft_internal.h"

namespace glsfft {

// Device tables, generated in FP64 on the host once per context: the
// four-step twiddles divided by N1, e^{-2 pi i k1 n2 / N} / N1 at
// [k1*N1 + n2] (N = N1^2), and the real-form DFT operand images.
struct TcTables {
    float2 *tw1024 = nullptr, *tw4096 = nullptr;
    // the 32- and 64-point DFTs as tcgen05 B operands: FP16 hi then lo,
    // 128-byte-swizzled K-major images (tc5_fft.cu; 16 KB and 48 KB)
    unsigned char *dft32_sw = nullptr, *dft64_sw = nullptr;
    void *block = nullptr;  // one allocation holding all of the above
};

int tc_tables_create(TcTables *t);
void tc_tables_destroy(TcTables *t);

// 1-D FFTs of length n (1024 or 4096) of every row (rows = true) or column
// of `images` contiguous images, on tcgen05 (tc5_fft.cu); the line count
// must be a multiple of 4 resp. 2.
cudaError_t launch_tc_lines(int n, bool rows, const PassArgs &a, const TcTables &t, int images,
                            cudaStream_t s);
// Host: the N1-point DFT B operand image (N1 = 32: 16 KB, 64: 48 KB) from
// cos_sin[m] = {cos, sin}(2 pi m / N1).
void tc5_dft_image(int n1, const double (*cos_sin)[2], unsigned char *dst);

}  // namespace glsfft
