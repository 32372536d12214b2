// sched_internal.h -- the selectable schedules of the plain path's complex
// row and column passes, and the per-size choice a context keeps.
#pragma once
#include <cuda_runtime.h>

#include "fft_config.h"
#include "glsfft_internal.h"

namespace glsfft {

// id 0..kPassSchedules-1 of fft_config.h; unavailable ids give
// cudaErrorInvalidValue without launching
cudaError_t launch_rows_sched(int n, int id, const PassArgs &a, int images, cudaStream_t s);
cudaError_t launch_cols_sched(int n, int id, const PassArgs &a, int images, cudaStream_t s);

struct FftSchedule {
    int row = 0;  // schedule of the row pass (line length cols)
    int col = 0;  // schedule of the column pass (line length rows)
};
inline long long sched_key(int rows, int cols) { return ((long long)rows << 20) | cols; }

}  // namespace glsfft
