// fft_config.h -- tile shapes per line length N (power of two, 1..4096).
//
// Rows:    E complex per thread, LINES rows per 256-thread block.
// Columns: E complex per thread, W adjacent columns per block (W*8 bytes per
//          image row segment; >= 32 B so every DRAM sector fetched is used).
// POC:     like columns, but two lines live in registers at once.
#pragma once

namespace glsfft {

__host__ __device__ constexpr int cmin(int a, int b) { return a < b ? a : b; }
__host__ __device__ constexpr int cmax(int a, int b) { return a > b ? a : b; }

__host__ __device__ constexpr int rows_E(int n) { return cmin(n, 16); }
__host__ __device__ constexpr int rows_T(int n) { return n / rows_E(n); }
__host__ __device__ constexpr int rows_LINES(int n) { return cmax(1, 256 / rows_T(n)); }

__host__ __device__ constexpr int cols_E(int n) { return n == 4096 ? 32 : cmin(n, 16); }
__host__ __device__ constexpr int cols_T(int n) { return n / cols_E(n); }
__host__ __device__ constexpr int cols_W(int n) {
    return n >= 2048 ? 4 : n == 1024 ? 8 : n == 512 ? 16 : cmax(16, cmin(64, 256 / cols_T(n)));
}

__host__ __device__ constexpr int poc_E(int n) { return cmin(n, 16); }
__host__ __device__ constexpr int poc_T(int n) { return n / poc_E(n); }
// 4 columns (32-byte row segments) at 256, 512 and 2048 points: a
// phaseCorrelate image is one launch of a few hundred blocks at most, so
// more, smaller blocks spread it over more SMs
__host__ __device__ constexpr int poc_W(int n) {
    return n == 4096 ? 2 : n == 1024 ? 8 : n >= 256 ? 4 : cmax(16, cmin(64, 256 / poc_T(n)));
}

// shared-memory floats2 for `count` complex values with one pad per 16
__host__ __device__ constexpr int padded_count(int count) { return count + (count >> 4); }

// ------------------------------------------------ selectable pass schedules
// The complex row and column passes of the plain path have kPassSchedules
// alternative schedules per line length; the autotuner times them and keeps
// the fastest per image size.  Schedule 0 is the fixed shape above.
//   1: half the elements per thread (radix bound lowered to E), twice the
//      threads per line
//   2: twice the elements per thread (radix <= 16, two butterflies per
//      thread per pass), half the threads per line
//   3: half the lines (rows) or columns (cols) per block
//   4: twice the lines or columns per block
//   5: 1 and 3 together (half the elements per thread, half the lines or
//      columns per block: smaller blocks, more of them resident per SM)
//   6: streamed column pass (fft_stream.cu): one persistent block per SM
//      that copies the next 128 KB tile in with the TMA while it transforms
//      the current one; 2048- and 4096-point columns only, bit-identical to
//      schedule 0
// Schedules 1..5 exist for N >= kSchedMinLen when the block has 32..1024
// threads, fits 227 KB of shared memory and its E divides N; every
// schedule computes the same transform (the rounding differs with the radix
// order, within the FP32 error bound).
constexpr int kPassSchedules = 7;
constexpr int kSchedStreamed = 6;
constexpr int kSchedMinLen = 64;

struct PassShape {
    int E, MB, G;  // elements per thread, log2 radix bound, lines or columns per block
};

__host__ __device__ constexpr int ilog2s(int n) { return n <= 1 ? 0 : 1 + ilog2s(n >> 1); }

__host__ __device__ constexpr PassShape shape_variant(PassShape d, int id) {
    return id == 1 ? PassShape{d.E / 2, cmin(4, ilog2s(d.E / 2)), d.G}
         : id == 2 ? PassShape{d.E * 2, 4, d.G}
         : id == 3 ? PassShape{d.E, 4, d.G / 2}
         : id == 4 ? PassShape{d.E, 4, d.G * 2}
         : id == 5 ? PassShape{d.E / 2, cmin(4, ilog2s(d.E / 2)), d.G / 2}
                   : d;
}
__host__ __device__ constexpr PassShape row_shape(int n, int id) {
    return shape_variant(PassShape{rows_E(n), 4, rows_LINES(n)}, id);
}
__host__ __device__ constexpr PassShape col_shape(int n, int id) {
    return shape_variant(PassShape{cols_E(n), 4, cols_W(n)}, id);
}
// threads per block of a shape
__host__ __device__ constexpr int shape_threads(int n, PassShape s) { return s.G * (n / s.E); }
// shared-memory bytes of a shape (0 when the line needs one pass)
__host__ __device__ constexpr long shape_smem(int n, PassShape s, bool cols) {
    return (ilog2s(n) <= s.MB) ? 0
           : cols ? 8L * padded_count(n * s.G)
                  : 8L * s.G * padded_count(n);
}
__host__ __device__ constexpr bool shape_ok(int n, PassShape s, bool cols) {
    return s.G >= 1 && s.E >= 2 && s.E <= 32 && s.E <= n && n % s.E == 0 &&
           (1 << cmin(s.MB, ilog2s(n))) <= s.E && shape_threads(n, s) >= 32 &&
           shape_threads(n, s) <= 1024 && shape_smem(n, s, cols) <= 227L * 1024;
}
__host__ __device__ constexpr bool same_shape(PassShape a, PassShape b) {
    return a.E == b.E && a.MB == b.MB && a.G == b.G;
}
// whether schedule `id` of a row (cols=false) or column pass of length n
// exists and differs from schedule 0
__host__ __device__ constexpr bool sched_available(int n, int id, bool cols) {
    return id == 0 || (id == kSchedStreamed && cols && (n == 2048 || n == 4096)) ||
           (id > 0 && id < kSchedStreamed && n >= kSchedMinLen && n <= 4096 &&
            shape_ok(n, cols ? col_shape(n, id) : row_shape(n, id), cols) &&
            !same_shape(cols ? col_shape(n, id) : row_shape(n, id),
                        cols ? col_shape(n, 0) : row_shape(n, 0)));
}

}  // namespace glsfft
