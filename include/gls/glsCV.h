/*
 * gls/glsCV.h -- the C++ drop-in layer of the GB300 FFT path, mirroring the
 * reference's OpenCV-style API (glsCV/glsMat.h, glsFft.h, glsPhaseCorrelate.h,
 * glsCV.h) over device memory instead of GL textures.  Every call goes
 * through the C ABI of <glsfft.h>; a non-zero status becomes gls::Exception,
 * as GLS_Assert/CV_Assert throw cv::Exception in the reference
 * (glsCV/glsMacro.h:40).
 *
 * OpenCV itself is not required: the few value types the API needs (Size,
 * Point, Point2d, a continuous host Mat) and the type codes are defined here
 * with OpenCV's numeric values, in namespace gls.
 */
#ifndef GLS_GLSCV_H_
#define GLS_GLSCV_H_

#include <cstddef>
#include <cstdint>
#include <memory>
#include <stdexcept>
#include <string>
#include <vector>

#include "glsfft.h"

#if defined(__GNUC__)
#define GLS_EXPORT __attribute__((visibility("default")))
#else
#define GLS_EXPORT
#endif

namespace gls {

// OpenCV type codes and flags (same values as OpenCV 3.1).
enum { CV_32F = 5, CV_32FC1 = 5, CV_32FC2 = 13 };
enum { DFT_INVERSE = 1, DFT_SCALE = 2 };
// glsCV/glsFft.h:43-47
enum { GLS_FFT_SCALE = DFT_SCALE, GLS_FFT_INVERSE = DFT_INVERSE, GLS_FFT_SHIFT = 64 };
enum { NORM_INF = 1, NORM_L1 = 2, NORM_L2 = 4, NORM_MINMAX = 32 };  // OpenCV values

inline int cv_depth(int type) { return type & 7; }
inline int cv_channels(int type) { return (type >> 3) + 1; }
inline size_t cv_elem_size(int type) { return (size_t)4 * (size_t)cv_channels(type); }

struct Size {
    int width = 0, height = 0;
    Size() {}
    Size(int w, int h) : width(w), height(h) {}
    bool operator==(const Size &o) const { return width == o.width && height == o.height; }
    bool operator!=(const Size &o) const { return !(*this == o); }
};
struct Point {
    int x = 0, y = 0;
    Point() {}
    Point(int x_, int y_) : x(x_), y(y_) {}
};
struct Point2d {
    double x = 0, y = 0;
    Point2d() {}
    Point2d(double x_, double y_) : x(x_), y(y_) {}
};

// Thrown where the reference throws cv::Exception.
class GLS_EXPORT Exception : public std::runtime_error {
  public:
    Exception(int status, const std::string &where);
    int status() const { return status_; }

  private:
    int status_;
};

// Continuous host image (the role cv::Mat plays in the reference API).
class GLS_EXPORT Mat {
  public:
    int rows = 0, cols = 0;
    Mat() {}
    Mat(Size s, int type);
    Mat(int rows_, int cols_, int type);
    int type() const { return type_; }
    int channels() const { return cv_channels(type_); }
    int depth() const { return cv_depth(type_); }
    Size size() const { return Size(cols, rows); }
    size_t total() const { return (size_t)rows * cols; }
    bool empty() const { return total() == 0; }
    size_t bytes() const { return total() * cv_elem_size(type_); }
    template <class T> T *ptr(int r = 0) { return reinterpret_cast<T *>(data_.data()) + (size_t)r * cols * channels(); }
    template <class T> const T *ptr(int r = 0) const {
        return reinterpret_cast<const T *>(data_.data()) + (size_t)r * cols * channels();
    }
    void *data() { return data_.data(); }
    const void *data() const { return data_.data(); }

  private:
    int type_ = CV_32FC1;
    std::vector<unsigned char> data_;
};

// Refcounted device image, glsCV/glsMat.h:45-165: assignment is shallow
// (glsMat.cpp:101-117), clone()/copyTo() deep; upload/download synchronous.
class GLS_EXPORT GlsMat {
  public:
    int rows = 0, cols = 0;

    GlsMat() {}
    GlsMat(const Size size, const int type);
    explicit GlsMat(const Mat &host);

    int type() const { return type_; }
    int channels() const { return cv_channels(type_); }
    int depth() const { return cv_depth(type_); }
    Size size() const { return Size(cols, rows); }
    size_t total() const { return (size_t)rows * cols; }
    bool empty() const { return !buf_; }
    bool isContinuous() const { return true; }

    void upload(const Mat &src);
    void download(Mat &dst) const;
    operator Mat() const;
    GlsMat clone() const;
    void copyTo(GlsMat &m) const;

    // device address of the pixels (row-major, continuous)
    void *devptr() const;
    // true when both refer to the same device storage
    bool shares(const GlsMat &o) const { return buf_ && buf_ == o.buf_; }

  private:
    struct Buffer;
    std::shared_ptr<Buffer> buf_;
    int type_ = CV_32FC1;
};

// glsCV/glsCV.h:67-68.  Creates the process-wide context on a CUDA device
// (the reference creates a hidden GL window); calls below create it lazily.
GLS_EXPORT void glsCvInit(int device = 0);
GLS_EXPORT void glsCvTerminate();
// The context the gls:: functions use (for mixing with the C ABI).
GLS_EXPORT glsfft_context glsCvContext();

// glsCV/glsFft.h:55.  src: CV_32FC1 or CV_32FC2, power-of-two rows and cols
// (square, rectangular or 1-D); dst becomes CV_32FC2 of the same size and
// reuses its storage when it already has that size and type (in place when
// it is src), as getDstMat does (glsCV/glsMat.h:205-213).
GLS_EXPORT void fft(const GlsMat &src, GlsMat &dst, int flag = 0);
// Convenience (not in the reference): fft with GLS_FFT_INVERSE added.
GLS_EXPORT void ifft(const GlsMat &src, GlsMat &dst, int flag = 0);

// glsCV/glsPhaseCorrelate.h:58: shift of src2 relative to src1 (both
// CV_32FC1, same power-of-two size), window CV_32FC1 of that size or empty.
GLS_EXPORT Point2d phaseCorrelate(const GlsMat &src1, const GlsMat &src2, GlsMat &window,
                                  double *response = 0);
// Same with an explicit centroid box (the reference fixes 5, :219).
GLS_EXPORT Point2d phaseCorrelate(const GlsMat &src1, const GlsMat &src2, GlsMat &window,
                                  double *response, int box);

// Extensions (not in the reference): the same operations computed with the
// reference's own CPU Stockham arithmetic -- algo 0: the radix-2 type1
// routine, 1: the radix-4 routine per line (the shader's algorithm) -- so the
// results are bit-identical to it (glsfft_fft2d_reference,
// glsfft_phase_correlate_reference).  fftReference takes CV_32FC2 only.
GLS_EXPORT void fftReference(const GlsMat &src, GlsMat &dst, int flag = 0, int algo = 0);
GLS_EXPORT Point2d phaseCorrelateReference(const GlsMat &src1, const GlsMat &src2,
                                           GlsMat &window, double *response = 0,
                                           int algo = 0);

// glsCV/glsBasicOperation.h:78-88: CV_32FC2 spectra; dst is (re)allocated
// like getDstMat does (CV_32FC2 for the products, CV_32FC1 for magnitudes).
GLS_EXPORT void mulSpectrums(const GlsMat &src0, const GlsMat &src1, GlsMat &dst,
                             bool conj = false);
GLS_EXPORT void mulSpectrumsPhaseOnly(const GlsMat &src0, const GlsMat &src1, GlsMat &dst);
GLS_EXPORT void magSpectrums(const GlsMat &src, GlsMat &dst);
GLS_EXPORT void logMagSpectrums(const GlsMat &src, GlsMat &dst, float offset);

// glsCV/glsMinMaxLoc.h:42: CV_32FC1; first occurrence in row-major order.
// The mask must be empty, as in the reference (glsMinMaxLoc.cpp:153).
GLS_EXPORT void minMaxLoc(const GlsMat &src, double *minVal, double *maxVal = 0,
                          Point *minLoc = 0, Point *maxLoc = 0, const GlsMat &mask = GlsMat());

// glsCV/glsNormalize.h:47: CV_32FC1.  NORM_MINMAX (dst in [alpha, beta]) is
// implemented; NORM_L1 / NORM_L2 throw (they need gls::norm, outside this path).
GLS_EXPORT void normalize(const GlsMat &src, GlsMat &dst, double alpha = 1, double beta = 0,
                          int normType = NORM_L2);

}  // namespace gls

#endif  // GLS_GLSCV_H_
