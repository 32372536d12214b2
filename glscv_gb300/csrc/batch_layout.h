// batch_layout.h -- index arithmetic of the batch plans' tiles and of the
// column-tiled workspace, shared by the persistent kernel (device) and the
// host-side plan and its unit test (plain C++, no CUDA headers needed).
#pragma once

#if defined(__CUDACC__)
#define GLSFFT_HD __host__ __device__
#else
#define GLSFFT_HD
#endif

namespace glsfft {

constexpr int kBatchTileElems = 4096;  // complex values per tile (16 per compute thread)

// Rows of the shortest columns that get the column-tiled workspace: with
// 1024-point columns a columns tile is W = 4 columns, 32-byte segments of
// 1024 rows through the column map; shorter columns have wider tiles
// (64..512-byte segments) that the map already reads well, and the extra
// buffer only adds traffic (measured on GB300: 512 uneven images of 128^2 ..
// 1024^2, forward, 0.749 ms with a workspace for every shape against 0.739
// without).
constexpr int kBatchTiledMinRows = 1024;

// Whether an image of this shape uses the column-tiled workspace: whole
// tiles both ways and one rows tile = one tensor box (W, cols / W, lines),
// every box dimension <= 256.
GLSFFT_HD constexpr bool batch_tiled_ok(int rows, int cols) {
    return rows >= kBatchTiledMinRows && cols >= 16 && rows <= 1024 &&
           (long long)rows * cols >= kBatchTileElems && (long long)rows * cols <= 256LL * kBatchTileElems;
}

// Whether the image keeps every intermediate in its workspace
// (BatchImage::ws_inplace): a rows tile is 256 pieces of exactly 128 bytes.
GLSFFT_HD constexpr bool batch_tiled_inplace(int rows, int cols) {
    return batch_tiled_ok(rows, cols) && (long long)rows * cols == 256LL * kBatchTileElems;
}

// Column-tiled layout of a rows x cols image, W = kBatchTileElems / rows
// columns per tile: pixel (r, c) at ((c / W) * rows + r) * W + c % W, so
// columns tile j is the rows * W pixels from j * rows * W on.
GLSFFT_HD constexpr long long batch_tiled_index(int rows, int r, int c) {
    const int w = kBatchTileElems / rows;
    return ((long long)(c / w) * rows + r) * w + c % w;
}

// Stage position of value t (column t, thread t of the line) of line `l`
// of an n-point rows tile loaded as one in-place workspace box (n >= 1024,
// rows = 2^20 / n): piece j = column / W (W = n / 256) holds the W values of
// columns tile j of the tile's 4096 / n lines, 16 values = 128 bytes, whose
// 16-byte chunks the 128-byte swizzle permutes by j % 8.  Column
// t + m * (n / 16) lies in piece t / W + 16 m, at this position + 256 m (the
// swizzle acts on bits 1-3 only).
GLSFFT_HD constexpr unsigned ws_swz_base(unsigned n, unsigned l, unsigned t) {
    const unsigned w = n / 256, j = t / w;
    return (j * 16 + l * w + t % w) ^ ((j & 7) << 1);
}

}  // namespace glsfft
