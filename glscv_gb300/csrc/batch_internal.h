// batch_internal.h -- data shared by the persistent batched FFT kernel and its
// host-side plan (batch.cu).  Not a public header.
#pragma once
#include <cuda_runtime.h>
#include <stdint.h>

#include "batch_layout.h"

namespace glsfft {

constexpr int kBatchThreads = 256;      // threads of a persistent block
constexpr int kBatchMaxPasses = 4;      // passes per image (2 transforms)

// One image of a batch plan.  Pass 0 reads src; every later pass reads and
// writes dst (in place), so src may equal dst.
//
// When `work` is set (the warp-specialised kernel; images that
// batch_tiled_ok accepts), a rows pass writes its result to `work` in
// the column-tiled layout instead of to dst, and the columns pass that
// follows reads its tile from there as one contiguous block and writes dst.
// Column-tiled layout: with W = kBatchTileElems / rows columns per tile,
// pixel (r, c) is at work[((c / W) * rows + r) * W + c % W] -- a columns
// tile is rows * W consecutive pixels, and the W-wide pieces of one row are
// rows * W apart.  Two ways to use it:
//   * `ws_inplace` = 0: every rows pass reads rows (src, then dst) and
//     stores its tile into work with one 3-D tensor box; every columns pass
//     reads work and writes dst.  No pass reads a buffer it writes.
//   * `ws_inplace` = 1 (rows * cols = 2^20: 1024^2, where the L = 4 rows
//     of a rows tile make one 128-byte piece in every columns tile): every
//     intermediate stays in work.  Rows passes store through the 3-D box
//     as above; a later rows pass loads its tile as one 2-D tensor box of
//     256 such pieces (128-byte swizzle: piece j's 16-byte chunks permuted
//     by j % 8), so the rows kernel reads that stage in box order; columns
//     passes read and write their block in place; only pass 0 reads src and
//     only the last columns pass writes dst.
// Either way src may equal dst (pass 0 completes before dst is written).
struct BatchImage {
    const float2 *src;
    float2 *dst;
    float2 *work;              // column-tiled workspace, or null
    int rows, cols;
    int row_tiles, col_tiles;  // tiles of a rows pass / a columns pass
    int ws_inplace;            // 1: the intermediates stay in work (see above)
    int pad;
};

// One pass of the chain every image runs through.
struct BatchPass {
    int along_rows;  // 1: 1-D FFT of every row, 0: of every column
    unsigned flags;  // PF_CONJ_IN / PF_CONJ_OUT / PF_SHIFT_ROWS / PF_SHIFT_COLS
    int scale;       // 1: multiply by 1/length
    int pad;
};

// Work item: image, pass, tile, and how many tiles of the previous pass of
// the same image must be complete first (0 for pass 0).
struct BatchItem {
    int image;
    int pass;
    int tile;
    int need;
};

struct BatchArgs {
    const BatchImage *images;
    const BatchPass *passes;
    const BatchItem *items;
    int n_items;
    int n_passes;
    unsigned *head;        // next item index (zeroed before each launch)
    unsigned *done;        // [image * kBatchMaxPasses + pass] completed tiles (zeroed)
    int *error;            // set to a non-zero code when a bounded wait expires
    const float2 *tw;      // twiddle tables (entries [n, 2n) for length n)
    long long wait_limit_ns;  // bound on one dependency wait
    const void *tmaps;     // warp-specialised kernel: two 128-B CUtensorMaps per image
                           // (kBatchTmapsPerImage): the column map of dst, the tiled map of work
    int claim_chunk;       // warp-specialised kernel: items claimed per queue atomic (1..4)
    int claim_ahead;       // 1: claim the next chunk before working on the current one
    unsigned long long *stats;  // warp-specialised kernel: kBatchStats timing sums, or null
};

// Timing sums (nanoseconds, %globaltimer) a warp-specialised launch adds
// when BatchArgs::stats is set: per block, producer time in dependency
// waits, in waits for a stage to be free (compute done + store read), in
// store-completion waits before publishing, and its whole run; compute
// warp 0's waits for staged tiles and its whole run; items issued.
enum {
    BS_DEP_WAIT = 0,
    BS_REFILL_WAIT,
    BS_PUBLISH_WAIT,
    BS_PRODUCER_TOTAL,
    BS_FULL_WAIT,
    BS_COMPUTE_TOTAL,
    BS_ITEMS,
    BS_BLOCKS,
    kBatchStats
};

// Persistent kernel variants: plain (every thread loads and stores its
// operands) and warp-specialised (a producer warp stages tiles with TMA into
// a shared-memory ring, eight compute warps run the FFT and leave the results
// in the stage, the producer stores them with TMA): 1 or 2 blocks per SM
// with 3 stages, or 3 blocks per SM with 2 stages.
enum { BATCH_PLAIN = 0, BATCH_TMA_WS1 = 1, BATCH_TMA_WS2 = 2, BATCH_TMA_WS3 = 3 };

cudaError_t launch_batch_persistent(const BatchArgs &a, int grid, cudaStream_t s);
int batch_persistent_grid(int device);  // blocks that fit on the device at once
bool batch_supported(int rows, int cols);

cudaError_t launch_batch_ws(const BatchArgs &a, int grid, int blocks_per_sm, cudaStream_t s);
int batch_ws_grid(int device, int blocks_per_sm);

// Build the 2-D tensor map (8-byte elements, box W x min(rows, 256)) that the
// warp-specialised kernel uses to stage column tiles of `img` (rows x cols).
int make_column_tmap(void *tmap128, const void *img, int rows, int cols);

// Tensor maps per image in BatchArgs::tmaps: [0] the column map of dst,
// [1] the 3-D tiled map of work, [2] the swizzled 2-D map of an in-place
// image's work (zeroed where unused).
constexpr int kBatchTmapsPerImage = 3;

// Build a tensor map through which a rows pass moves one tile of the
// column-tiled layout of `work` (rows x cols).  `swizzled` = false: 3-D,
// dimensions (W, cols / W, rows) with strides (8, rows * W * 8, W * 8)
// bytes, box (W, cols / W, 4096 / cols) -- the box lands in shared memory as
// the tile's rows, one after another.  `swizzled` = true (in-place images
// only): 2-D, dimensions (rows * W, cols / W) with stride rows * W * 8
// bytes, box (16, 256), 128-byte swizzle -- a box is the tile's 256 pieces
// of 128 bytes, piece j's 16-byte chunk c at chunk c ^ (j % 8).
int make_tiled_tmap(void *tmap128, const void *work, int rows, int cols, bool swizzled);

}  // namespace glsfft
