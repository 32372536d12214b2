// Host unit test of the batch plans' column-tiled workspace arithmetic
// (glscv_gb300/csrc/batch_layout.h), compiled without CUDA.  The boxes the
// kernel moves are emulated element by element from their tensor-map
// definitions (batch.cpp: make_tiled_tmap) and checked against the index
// arithmetic the kernel uses.
#include <cstdio>
#include <cstdlib>
#include <vector>

#include "batch_layout.h"

using namespace glsfft;

static int failures = 0;
#define CHECK(c)                                                   \
    do {                                                           \
        if (!(c)) {                                                \
            std::printf("FAIL line %d: %s\n", __LINE__, #c);        \
            if (++failures > 20) std::exit(1);                     \
        }                                                          \
    } while (0)

int main() {
    // which shapes get a workspace, and which keep every intermediate there
    CHECK(batch_tiled_ok(1024, 1024) && batch_tiled_inplace(1024, 1024));
    CHECK(batch_tiled_ok(1024, 512) && !batch_tiled_inplace(1024, 512));
    CHECK(batch_tiled_ok(1024, 16) && !batch_tiled_ok(1024, 8));
    CHECK(!batch_tiled_ok(1024, 2048) && !batch_tiled_ok(512, 512) && !batch_tiled_ok(2048, 64));

    for (int cols : {16, 64, 512, 1024}) {
        const int rows = 1024, w = kBatchTileElems / rows, lines = kBatchTileElems / cols;
        const long long n = (long long)rows * cols;
        // the layout is a permutation; columns tile j is one contiguous block
        std::vector<int> hit(n, 0);
        for (int r = 0; r < rows; r++)
            for (int c = 0; c < cols; c++) {
                const long long i = batch_tiled_index(rows, r, c);
                CHECK(i >= 0 && i < n);
                if (i >= 0 && i < n) hit[i]++;
                CHECK(i / ((long long)rows * w) == c / w);
            }
        for (long long i = 0; i < n; i++) CHECK(hit[i] == 1);
        // 3-D box of rows tile k: dimensions (W, cols / W, rows), strides
        // (8, rows * W * 8, W * 8) bytes, box (W, cols / W, lines), traversed
        // innermost first into consecutive shared-memory slots: the stage
        // must hold the tile's rows in order
        for (int k = 0; k < rows / lines; k += 7) {
            long long slot = 0;
            for (int l = 0; l < lines; l++)
                for (int j = 0; j < cols / w; j++)
                    for (int x = 0; x < w; x++, slot++) {
                        const long long g = (long long)j * rows * w + (long long)(k * lines + l) * w + x;
                        CHECK(g == batch_tiled_index(rows, k * lines + l, j * w + x));
                        CHECK(slot == (long long)l * cols + j * w + x);
                    }
        }
    }

    // 2-D swizzled box of an in-place 1024^2 rows tile k: dimensions
    // (rows * W, cols / W), box (16, 256), 128-byte swizzle: box element
    // (x, j) lands at byte 128 j + 16 ((x / 2) ^ (j % 8)) + 8 (x % 2) of a
    // 1024-byte-aligned stage.  Thread t of line l must find column
    // t + 64 m at ws_swz_base + 256 m.
    {
        const unsigned n = 1024, rows = 1024, w = 4, lines = 4, T = n / 16;
        std::vector<long long> slot_of_pixel((size_t)lines * n, -1);
        const int k = 37;  // any rows tile
        for (unsigned j = 0; j < 256; j++)
            for (unsigned x = 0; x < 16; x++) {
                const long long g = (long long)j * rows * w + (long long)k * 16 + x;
                const unsigned slot = j * 16 + (((x / 2) ^ (j % 8)) * 2) + (x % 2);
                // the pixel at tiled index g
                const unsigned l = x / w, c = j * w + x % w;
                CHECK(g == batch_tiled_index(rows, k * lines + l, c));
                slot_of_pixel[(size_t)l * n + c] = slot;
            }
        for (unsigned l = 0; l < lines; l++)
            for (unsigned t = 0; t < T; t++)
                for (unsigned m = 0; m < 16; m++)
                    CHECK(slot_of_pixel[(size_t)l * n + t + m * T] == (long long)(ws_swz_base(n, l, t) + 256 * m));
    }

    if (failures) return 1;
    std::printf("ALL OK\n");
    return 0;
}
