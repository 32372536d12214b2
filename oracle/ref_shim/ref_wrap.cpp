/*
 * extern "C" entry points around glsCV's own CPU Stockham routines
 * (UnitTest_glsCV/fft_stockhum.cpp), so tests can call the reference code
 * through ctypes.  Built only by oracle/build_ref.sh into oracle/_ref.
 * Test infrastructure: the product library never links this.
 */
#include "stdafx.h"

void fft_dit_Stockham_radix2_type1(const Mat &src, Mat &dst); /* fft_stockhum.cpp:436 */
void fft_dit_Stockham_radix4_type0(const Mat &src, Mat &dst); /* fft_stockhum.cpp:771 */
void fft_dif_Stockham_radix4_type0(const Mat &src, Mat &dst); /* fft_stockhum.cpp:597 */

static Mat to_mat(const float *in, int rows, int cols) {
    Mat m(Size(cols, rows), CV_32FC2);
    std::memcpy(m.data(), in, sizeof(float) * 2 * (size_t)rows * cols);
    return m;
}

static void from_mat(Mat &m, float *out) {
    std::memcpy(out, m.data(), sizeof(float) * 2 * (size_t)m.rows * m.cols);
}

extern "C" {

/* Square N x N, radix-2 DIT type1 (OpenMP over rows / columns). */
int ref_fft_r2t1_square(const float *in, float *out, int n) {
    try {
        Mat src = to_mat(in, n, n), dst;
        fft_dit_Stockham_radix2_type1(src, dst);
        from_mat(dst, out);
        return 0;
    } catch (...) {
        return -1;
    }
}

/* Square N x N, radix-4 DIF (recursive, with transposes). */
int ref_fft_dif_r4_square(const float *in, float *out, int n) {
    try {
        Mat src = to_mat(in, n, n), dst;
        fft_dif_Stockham_radix4_type0(src, dst);
        from_mat(dst, out);
        return 0;
    } catch (...) {
        return -1;
    }
}

/*
 * Radix-4 DIT (the GLSL shader's algorithm) on every row, then every column,
 * each as its own 1 x N / N x 1 call, which is how that routine is correct
 * for every shape.  rows, cols >= 4.
 */
int ref_fft_r4_lines(const float *in, float *out, int rows, int cols) {
    try {
        std::vector<float> img(in, in + 2 * (size_t)rows * cols);
        if (cols > 1)
            for (int r = 0; r < rows; r++) {
                Mat line = to_mat(&img[2 * (size_t)r * cols], 1, cols), res;
                fft_dit_Stockham_radix4_type0(line, res);
                from_mat(res, &img[2 * (size_t)r * cols]);
            }
        if (rows > 1) {
            std::vector<float> col(2 * (size_t)rows);
            for (int c = 0; c < cols; c++) {
                for (int r = 0; r < rows; r++) {
                    col[2 * r] = img[2 * ((size_t)r * cols + c)];
                    col[2 * r + 1] = img[2 * ((size_t)r * cols + c) + 1];
                }
                Mat line = to_mat(col.data(), rows, 1), res;
                fft_dit_Stockham_radix4_type0(line, res);
                from_mat(res, col.data());
                for (int r = 0; r < rows; r++) {
                    img[2 * ((size_t)r * cols + c)] = col[2 * r];
                    img[2 * ((size_t)r * cols + c) + 1] = col[2 * r + 1];
                }
            }
        }
        std::memcpy(out, img.data(), sizeof(float) * img.size());
        return 0;
    } catch (...) {
        return -1;
    }
}

} /* extern "C" */
