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
__host__ __device__ constexpr int poc_W(int n) {
    return n == 4096 ? 2 : n == 2048 ? 4 : n == 1024 ? 8 : n == 512 ? 16 : cmax(16, cmin(64, 256 / poc_T(n)));
}

// shared-memory floats2 for `count` complex values with one pad per 16
__host__ __device__ constexpr int padded_count(int count) { return count + (count >> 4); }

}  // namespace glsfft
