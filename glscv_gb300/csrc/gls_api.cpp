// gls_api.cpp -- the C++ drop-in layer (include/gls/glsCV.h) over the C ABI.
#include "gls/glsCV.h"

#include <cuda_runtime.h>

#include <mutex>
#include <string>

namespace gls {

Exception::Exception(int status, const std::string &where)
    : std::runtime_error(where + ": " + glsfft_status_string(status)), status_(status) {}

namespace {

std::mutex g_ctx_mutex;
glsfft_context g_ctx = nullptr;

void check(int status, const char *where) {
    if (status != GLSFFT_SUCCESS) throw Exception(status, where);
}
void check_cuda(cudaError_t e, const char *where) {
    if (e != cudaSuccess) {
        cudaGetLastError();
        throw Exception(GLSFFT_ERROR_CUDA, std::string(where) + " (" + cudaGetErrorString(e) + ")");
    }
}
void assert_that(bool ok, const char *what) {
    if (!ok) throw Exception(GLSFFT_ERROR_INVALID_VALUE, what);
}

glsfft_context context() {
    std::lock_guard<std::mutex> lock(g_ctx_mutex);
    if (!g_ctx) check(glsfft_context_create(&g_ctx, 0), "glsCvInit");
    return g_ctx;
}

}  // namespace

// ------------------------------------------------------------------ Mat
Mat::Mat(Size s, int type) : rows(s.height), cols(s.width), type_(type) {
    data_.assign((size_t)s.width * s.height * cv_elem_size(type), 0);
}
Mat::Mat(int rows_, int cols_, int type) : Mat(Size(cols_, rows_), type) {}

// --------------------------------------------------------------- GlsMat
struct GlsMat::Buffer {
    void *ptr = nullptr;
    size_t bytes = 0;
    explicit Buffer(size_t n) : bytes(n) {
        context();  // device selected by glsCvInit
        check_cuda(cudaMalloc(&ptr, n ? n : 1), "GlsMat allocation");
    }
    ~Buffer() {
        if (ptr) cudaFree(ptr);
    }
};

GlsMat::GlsMat(const Size size, const int type) : rows(size.height), cols(size.width), type_(type) {
    assert_that(size.width > 0 && size.height > 0, "GlsMat: empty size");
    buf_ = std::make_shared<Buffer>(total() * cv_elem_size(type));
}

GlsMat::GlsMat(const Mat &host) : GlsMat(host.size(), host.type()) { upload(host); }

void *GlsMat::devptr() const { return buf_ ? buf_->ptr : nullptr; }

void GlsMat::upload(const Mat &src) {
    if (empty() || src.size() != size() || src.type() != type()) *this = GlsMat(src.size(), src.type());
    check_cuda(cudaMemcpy(buf_->ptr, src.data(), src.bytes(), cudaMemcpyHostToDevice), "GlsMat::upload");
}

void GlsMat::download(Mat &dst) const {
    assert_that(!empty(), "GlsMat::download: empty");
    if (dst.size() != size() || dst.type() != type()) dst = Mat(size(), type());
    check_cuda(cudaMemcpy(dst.data(), buf_->ptr, dst.bytes(), cudaMemcpyDeviceToHost),
               "GlsMat::download");
}

GlsMat::operator Mat() const {
    Mat m;
    download(m);
    return m;
}

GlsMat GlsMat::clone() const {
    GlsMat m;
    copyTo(m);
    return m;
}

void GlsMat::copyTo(GlsMat &m) const {
    assert_that(!empty(), "GlsMat::copyTo: empty");
    if (m.empty() || m.size() != size() || m.type() != type() || m.shares(*this))
        m = GlsMat(size(), type());
    check_cuda(cudaMemcpy(m.buf_->ptr, buf_->ptr, buf_->bytes, cudaMemcpyDeviceToDevice),
               "GlsMat::copyTo");
}

// ------------------------------------------------------------- context
void glsCvInit(int device) {
    std::lock_guard<std::mutex> lock(g_ctx_mutex);
    if (g_ctx) return;
    check_cuda(cudaSetDevice(device), "glsCvInit");
    check(glsfft_context_create(&g_ctx, device), "glsCvInit");
}

void glsCvTerminate() {
    std::lock_guard<std::mutex> lock(g_ctx_mutex);
    if (g_ctx) glsfft_context_destroy(g_ctx);
    g_ctx = nullptr;
}

glsfft_context glsCvContext() { return context(); }

// ------------------------------------------------------------ outputs
// The output image of an operation, chosen before dst is assigned (dst may
// be the same object as a source, which must stay valid while it is read);
// the operation computes into it and assigns dst = out at the end, as the
// reference's `_dst = getDstMat(...); ...; dst = _dst;` does.
namespace {
// getDstMat (glsMat.h:205-213, the size / type form): dst's storage when it
// already has the size and type, else a new image
GlsMat out_for(const GlsMat &dst, Size size, int type) {
    if (dst.empty() || dst.size() != size || dst.type() != type) return GlsMat(size, type);
    return dst;
}
// getDstMat (glsMat.h:173-196, the source form): also a new image when dst
// shares storage with a source, so other copies of that source keep its data
GlsMat out_for(const GlsMat &dst, const GlsMat &src0, const GlsMat &src1, int type) {
    if (dst.shares(src0) || dst.shares(src1)) return GlsMat(src0.size(), type);
    return out_for(dst, src0.size(), type);
}
}  // namespace

// ------------------------------------------------------------------ fft
void fft(const GlsMat &src, GlsMat &dst, int flag) {
    // glsFft.cpp:676-681
    assert_that(!src.empty(), "gls::fft: empty src");
    assert_that(src.channels() == 2 || src.channels() == 1, "gls::fft: channels must be 1 or 2");
    assert_that(src.depth() == CV_32F, "gls::fft: depth must be CV_32F");
    glsfft_context ctx = context();
    // the output is chosen before dst is touched: dst may be the very object
    // src refers to (fft(C, C)), and src must stay valid while it is read
    GlsMat out = out_for(dst, src.size(), CV_32FC2);
    int st;
    if (src.channels() == 2)
        st = glsfft_fft2d_c2c(ctx, src.devptr(), out.devptr(), src.rows, src.cols, flag, nullptr);
    else
        st = glsfft_fft2d_r2c_promote(ctx, static_cast<const float *>(src.devptr()), out.devptr(),
                                      src.rows, src.cols, flag, nullptr);
    check(st, "gls::fft");
    dst = out;
}

void ifft(const GlsMat &src, GlsMat &dst, int flag) { fft(src, dst, flag | GLS_FFT_INVERSE); }

// ------------------------------------------------------- phaseCorrelate
Point2d phaseCorrelate(const GlsMat &src1, const GlsMat &src2, GlsMat &window, double *response,
                       int box) {
    // glsPhaseCorrelate.cpp:144-150
    assert_that(!src1.empty() && !src2.empty(), "gls::phaseCorrelate: empty input");
    assert_that(src1.type() == src2.type() && src1.type() == CV_32FC1,
                "gls::phaseCorrelate: inputs must be CV_32FC1");
    if (src1.size() != src2.size()) throw Exception(GLSFFT_ERROR_SHAPE, "gls::phaseCorrelate");
    if (!window.empty()) {
        assert_that(window.type() == CV_32FC1, "gls::phaseCorrelate: window must be CV_32FC1");
        if (window.size() != src1.size()) throw Exception(GLSFFT_ERROR_SHAPE, "gls::phaseCorrelate");
    }
    double dx = 0, dy = 0, res = 0;
    check(glsfft_phase_correlate(context(), static_cast<const float *>(src1.devptr()),
                                 static_cast<const float *>(src2.devptr()),
                                 window.empty() ? nullptr : static_cast<const float *>(window.devptr()),
                                 src1.rows, src1.cols, box, &dx, &dy, &res, nullptr),
          "gls::phaseCorrelate");
    if (response) *response = res;
    return Point2d(dx, dy);
}

Point2d phaseCorrelate(const GlsMat &src1, const GlsMat &src2, GlsMat &window, double *response) {
    return phaseCorrelate(src1, src2, window, response, 5);
}

// ----------------------------------------------- reference-arithmetic mode
void fftReference(const GlsMat &src, GlsMat &dst, int flag, int algo) {
    assert_that(!src.empty(), "gls::fftReference: empty src");
    assert_that(src.type() == CV_32FC2, "gls::fftReference: src must be CV_32FC2");
    GlsMat out = out_for(dst, src.size(), CV_32FC2);
    check(glsfft_fft2d_reference(context(), src.devptr(), out.devptr(), 1, src.rows, src.cols,
                                 flag, algo, nullptr),
          "gls::fftReference");
    dst = out;
}

Point2d phaseCorrelateReference(const GlsMat &src1, const GlsMat &src2, GlsMat &window,
                                double *response, int algo) {
    assert_that(!src1.empty() && !src2.empty(), "gls::phaseCorrelateReference: empty input");
    assert_that(src1.type() == src2.type() && src1.type() == CV_32FC1,
                "gls::phaseCorrelateReference: inputs must be CV_32FC1");
    if (src1.size() != src2.size())
        throw Exception(GLSFFT_ERROR_SHAPE, "gls::phaseCorrelateReference");
    if (!window.empty()) {
        assert_that(window.type() == CV_32FC1, "gls::phaseCorrelateReference: window must be CV_32FC1");
        if (window.size() != src1.size())
            throw Exception(GLSFFT_ERROR_SHAPE, "gls::phaseCorrelateReference");
    }
    double dx = 0, dy = 0, res = 0;
    check(glsfft_phase_correlate_reference(
              context(), static_cast<const float *>(src1.devptr()),
              static_cast<const float *>(src2.devptr()),
              window.empty() ? nullptr : static_cast<const float *>(window.devptr()), src1.rows,
              src1.cols, 5, algo, &dx, &dy, &res, nullptr),
          "gls::phaseCorrelateReference");
    if (response) *response = res;
    return Point2d(dx, dy);
}

// ------------------------------------------------------ spectrum operations
namespace {
void check_spectrum(const GlsMat &m, const char *where) {
    assert_that(!m.empty() && m.type() == CV_32FC2, where);
}
}  // namespace

void mulSpectrums(const GlsMat &src0, const GlsMat &src1, GlsMat &dst, bool conj) {
    // glsBasicOperation.cpp:320-326
    check_spectrum(src0, "gls::mulSpectrums: src0 must be CV_32FC2");
    check_spectrum(src1, "gls::mulSpectrums: src1 must be CV_32FC2");
    if (src0.size() != src1.size()) throw Exception(GLSFFT_ERROR_SHAPE, "gls::mulSpectrums");
    GlsMat out = out_for(dst, src0, src1, CV_32FC2);
    check(glsfft_mul_spectrums(context(), src0.devptr(), src1.devptr(), out.devptr(), src0.rows,
                               src0.cols, conj ? 1 : 0, nullptr),
          "gls::mulSpectrums");
    dst = out;
}

void mulSpectrumsPhaseOnly(const GlsMat &src0, const GlsMat &src1, GlsMat &dst) {
    // glsBasicOperation.cpp:329-335
    check_spectrum(src0, "gls::mulSpectrumsPhaseOnly: src0 must be CV_32FC2");
    check_spectrum(src1, "gls::mulSpectrumsPhaseOnly: src1 must be CV_32FC2");
    if (src0.size() != src1.size()) throw Exception(GLSFFT_ERROR_SHAPE, "gls::mulSpectrumsPhaseOnly");
    GlsMat out = out_for(dst, src0, src1, CV_32FC2);
    check(glsfft_mul_spectrums_phase_only(context(), src0.devptr(), src1.devptr(), out.devptr(),
                                          src0.rows, src0.cols, nullptr),
          "gls::mulSpectrumsPhaseOnly");
    dst = out;
}

void magSpectrums(const GlsMat &src, GlsMat &dst) {
    // glsBasicOperation.cpp:337-343
    check_spectrum(src, "gls::magSpectrums: src must be CV_32FC2");
    GlsMat out = out_for(dst, src.size(), CV_32FC1);  // a CV_32FC1 never shares a CV_32FC2
    check(glsfft_mag_spectrums(context(), src.devptr(), static_cast<float *>(out.devptr()),
                               src.rows, src.cols, nullptr),
          "gls::magSpectrums");
    dst = out;
}

void logMagSpectrums(const GlsMat &src, GlsMat &dst, float offset) {
    // glsBasicOperation.cpp:345-351
    check_spectrum(src, "gls::logMagSpectrums: src must be CV_32FC2");
    GlsMat out = out_for(dst, src.size(), CV_32FC1);
    check(glsfft_log_mag_spectrums(context(), src.devptr(), static_cast<float *>(out.devptr()),
                                   src.rows, src.cols, offset, nullptr),
          "gls::logMagSpectrums");
    dst = out;
}

void minMaxLoc(const GlsMat &src, double *minVal, double *maxVal, Point *minLoc, Point *maxLoc,
               const GlsMat &mask) {
    // glsMinMaxLoc.cpp:149-153
    assert_that(!src.empty() && src.type() == CV_32FC1, "gls::minMaxLoc: src must be CV_32FC1");
    assert_that(mask.empty(), "gls::minMaxLoc: masks are not implemented (as in the reference)");
    int lmin[2] = {0, 0}, lmax[2] = {0, 0};
    check(glsfft_min_max_loc(context(), static_cast<const float *>(src.devptr()), src.rows,
                             src.cols, minVal, maxVal, lmin, lmax, nullptr),
          "gls::minMaxLoc");
    if (minLoc) *minLoc = Point(lmin[0], lmin[1]);
    if (maxLoc) *maxLoc = Point(lmax[0], lmax[1]);
}

void normalize(const GlsMat &src, GlsMat &dst, double alpha, double beta, int normType) {
    // glsNormalize.cpp:52-68
    assert_that(!src.empty() && src.type() == CV_32FC1, "gls::normalize: src must be CV_32FC1");
    assert_that(normType == NORM_MINMAX, "gls::normalize: only NORM_MINMAX is implemented");
    GlsMat out(src.size(), CV_32FC1);  // the reference builds a new _dst and assigns it
    check(glsfft_normalize_minmax(context(), static_cast<const float *>(src.devptr()),
                                  static_cast<float *>(out.devptr()), src.rows, src.cols, alpha,
                                  beta, nullptr),
          "gls::normalize");
    dst = out;
}

}  // namespace gls
