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

// The schedules an image size runs until it is set or tuned otherwise,
// from measurements on GB300 (one 4096^2 image, per pass): schedule 2 for
// 2048- and 4096-point rows (4096: 61 us vs 69 us for schedule 0) and the
// streamed pass for 4096-point columns (85 us vs 97 us); other lengths run
// schedule 0.
inline FftSchedule default_schedule(int rows, int cols) {
    FftSchedule s{};
    if (cols == 2048 || cols == 4096) s.row = 2;
    if (rows == 4096) s.col = kSchedStreamed;
    return s;
}
template <class Map>
inline FftSchedule schedule_for(const Map &m, int rows, int cols) {
    const auto it = m.find(sched_key(rows, cols));
    return it != m.end() ? it->second : default_schedule(rows, cols);
}

}  // namespace glsfft
