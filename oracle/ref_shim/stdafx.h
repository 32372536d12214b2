/*
 * Minimal stand-in for the precompiled header that glsCV's
 * UnitTest_glsCV/fft_stockhum.cpp includes.  OpenCV is not available, so
 * this provides just the cv:: pieces that file touches: a refcounted,
 * continuous cv::Mat of CV_32FC2 with ptr<>/clone/size/type, cv::Vec2f with
 * + and -, cv::Size, CV_Assert and an in-place cv::transpose.  `cout` is a
 * sink, because the reference's radix-4 routines print every butterfly.
 *
 * Written for this project (test infrastructure); it is used only by
 * oracle/build_ref.sh to build oracle/_ref from the reference's own source.
 */
#pragma once
#include <cmath>
#include <complex>
#include <cstring>
#include <memory>
#include <ostream>
#include <stdexcept>
#include <vector>

namespace glsref_shim {
struct NullOut {
    template <class T> NullOut &operator<<(const T &) { return *this; }
    NullOut &operator<<(std::ostream &(*)(std::ostream &)) { return *this; }
};
static NullOut null_out;
} // namespace glsref_shim

using std::complex;
using std::endl;
using std::vector;
#define cout glsref_shim::null_out

#define CV_32FC2 13
#define CV_Assert(expr)                                                        \
    do {                                                                       \
        if (!(expr)) throw std::runtime_error("CV_Assert failed: " #expr);     \
    } while (0)

namespace cv {
struct Size {
    int width = 0, height = 0;
    Size() {}
    Size(int w, int h) : width(w), height(h) {}
};

struct Vec2f {
    float val[2];
    Vec2f() : val{0.f, 0.f} {}
    Vec2f(float a, float b) : val{a, b} {}
    float &operator[](int i) { return val[i]; }
    const float &operator[](int i) const { return val[i]; }
};
inline Vec2f operator+(const Vec2f &a, const Vec2f &b) { return Vec2f(a[0] + b[0], a[1] + b[1]); }
inline Vec2f operator-(const Vec2f &a, const Vec2f &b) { return Vec2f(a[0] - b[0], a[1] - b[1]); }

/* CV_32FC2 only: rows x cols of Vec2f, shared storage like cv::Mat. */
class Mat {
  public:
    int rows = 0, cols = 0;
    Mat() {}
    Mat(Size s, int type) : rows(s.height), cols(s.width), type_(type),
        data_(std::make_shared<std::vector<Vec2f>>((size_t)s.width * s.height)) {}
    Mat(int r, int c, int type) : Mat(Size(c, r), type) {}
    Size size() const { return Size(cols, rows); }
    int type() const { return type_; }
    Mat clone() const {
        Mat m(size(), type_);
        if (data_) *m.data_ = *data_;
        return m;
    }
    template <class T> T *ptr(int r) { return reinterpret_cast<T *>(&(*data_)[(size_t)r * cols]); }
    template <class T> T *ptr(int r, int c) {
        return reinterpret_cast<T *>(&(*data_)[(size_t)r * cols + c]);
    }
    template <class T> const T *ptr(int r) const {
        return reinterpret_cast<const T *>(&(*data_)[(size_t)r * cols]);
    }
    template <class T> const T *ptr(int r, int c) const {
        return reinterpret_cast<const T *>(&(*data_)[(size_t)r * cols + c]);
    }
    Vec2f *data() { return data_->data(); }

  private:
    int type_ = CV_32FC2;
    std::shared_ptr<std::vector<Vec2f>> data_;
};

inline void transpose(const Mat &src, Mat &dst) {
    Mat t(Size(src.rows, src.cols), src.type());
    for (int r = 0; r < src.rows; r++)
        for (int c = 0; c < src.cols; c++) *t.ptr<Vec2f>(c, r) = *src.ptr<Vec2f>(r, c);
    dst = t;
}
} // namespace cv

using namespace cv;
