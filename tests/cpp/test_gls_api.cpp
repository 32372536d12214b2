// C++ test of the drop-in gls:: API (include/gls/glsCV.h), written like the
// reference's own unit tests: random images through gls::fft and
// gls::phaseCorrelate, checked against a double-precision DFT and a known
// shift.  Built and run by tests/test_cpp_api.py.
#include <cmath>
#include <complex>
#include <cstdio>
#include <cstdlib>
#include <random>
#include <string>
#include <vector>

#include "gls/glsCV.h"

using gls::GlsMat;
using gls::Mat;
using gls::Size;

static int failures = 0;
#define EXPECT(cond, msg)                                                      \
    do {                                                                       \
        if (!(cond)) {                                                         \
            std::printf("FAIL %s:%d %s\n", __FILE__, __LINE__, msg);           \
            failures++;                                                        \
        }                                                                      \
    } while (0)

static Mat random_complex(int rows, int cols, unsigned seed) {
    Mat m(rows, cols, gls::CV_32FC2);
    std::mt19937 rng(seed);
    std::uniform_real_distribution<float> u(-1.f, 1.f);
    float *p = m.ptr<float>();
    for (size_t i = 0; i < m.total() * 2; i++) p[i] = u(rng);
    return m;
}

// separable DFT in double (rows then columns)
static std::vector<std::complex<double>> dft2(const Mat &m, int sign) {
    const int R = m.rows, C = m.cols;
    std::vector<std::complex<double>> a(m.total()), b(m.total());
    const float *p = m.ptr<float>();
    for (size_t i = 0; i < m.total(); i++) a[i] = {p[2 * i], p[m.channels() == 2 ? 2 * i + 1 : 0] * (m.channels() == 2)};
    if (m.channels() == 1)
        for (size_t i = 0; i < m.total(); i++) a[i] = {p[i], 0.0};
    const double pi = 3.14159265358979323846;
    for (int r = 0; r < R; r++)
        for (int k = 0; k < C; k++) {
            std::complex<double> s = 0;
            for (int n = 0; n < C; n++) s += a[(size_t)r * C + n] * std::polar(1.0, sign * 2 * pi * k * n / C);
            b[(size_t)r * C + k] = s;
        }
    for (int c = 0; c < C; c++)
        for (int k = 0; k < R; k++) {
            std::complex<double> s = 0;
            for (int n = 0; n < R; n++) s += b[(size_t)n * C + c] * std::polar(1.0, sign * 2 * pi * k * n / R);
            a[(size_t)k * C + c] = s;
        }
    return a;
}

static double rel_err(const Mat &got, const std::vector<std::complex<double>> &ref) {
    const float *p = got.ptr<float>();
    double num = 0, den = 0;
    for (size_t i = 0; i < got.total(); i++) {
        std::complex<double> g(p[2 * i], p[2 * i + 1]);
        num += std::norm(g - ref[i]);
        den += std::norm(ref[i]);
    }
    return std::sqrt(num / den);
}

static void test_fft() {
    for (auto shape : {std::make_pair(64, 64), std::make_pair(32, 128), std::make_pair(1, 256),
                       std::make_pair(128, 1)}) {
        Mat src = random_complex(shape.first, shape.second, 7u + shape.first);
        GlsMat g(src), f;
        gls::fft(g, f);
        Mat out = f;
        const double e = rel_err(out, dft2(src, -1));
        EXPECT(e < 1e-6, "forward fft vs double DFT");
        // round trip: inverse with scale
        GlsMat back;
        gls::fft(f, back, gls::GLS_FFT_INVERSE | gls::GLS_FFT_SCALE);
        Mat rt = back;
        double num = 0, den = 0;
        for (size_t i = 0; i < 2 * src.total(); i++) {
            const double d = rt.ptr<float>()[i] - src.ptr<float>()[i];
            num += d * d;
            den += (double)src.ptr<float>()[i] * src.ptr<float>()[i];
        }
        EXPECT(std::sqrt(num / den) < 1e-6, "round trip");
    }
    // 1-channel input is promoted with imag = 0 (glsFft.cpp:684-689)
    Mat real(32, 32, gls::CV_32FC1), cplx(32, 32, gls::CV_32FC2);
    for (size_t i = 0; i < real.total(); i++) {
        real.ptr<float>()[i] = (float)std::sin(0.37 * i);
        cplx.ptr<float>()[2 * i] = real.ptr<float>()[i];
        cplx.ptr<float>()[2 * i + 1] = 0.f;
    }
    GlsMat gr(real), gc(cplx), fr, fc;
    gls::fft(gr, fr);
    gls::fft(gc, fc);
    Mat a = fr, b = fc;
    bool same = true;
    for (size_t i = 0; i < 2 * a.total(); i++) same &= a.ptr<float>()[i] == b.ptr<float>()[i];
    EXPECT(same && fr.type() == gls::CV_32FC2, "CV_32FC1 promotion");
    // in place, and shallow copies share storage like the reference's textures
    Mat src = random_complex(64, 64, 99);
    GlsMat g(src), alias = g, deep = g.clone();
    gls::fft(g, g);
    Mat r1 = g, r2 = alias, r3 = deep;
    EXPECT(rel_err(r1, dft2(src, -1)) < 1e-6, "in-place fft");
    EXPECT(r1.ptr<float>()[5] == r2.ptr<float>()[5], "shallow copy shares storage");
    EXPECT(r3.ptr<float>()[5] == src.ptr<float>()[5], "clone is deep");
    // inverse convenience + SHIFT: quadrant swap of the spectrum
    GlsMat sh;
    gls::fft(GlsMat(src), sh, gls::GLS_FFT_SHIFT);
    Mat s1 = sh;
    auto ref = dft2(src, -1);
    const std::complex<double> dc(s1.ptr<float>()[2 * (32 * 64 + 32)], s1.ptr<float>()[2 * (32 * 64 + 32) + 1]);
    EXPECT(std::abs(dc - ref[0]) < 1e-3 * std::abs(ref[0]) + 1e-3, "SHIFT moves DC to the centre");
}

static void test_phase_correlate() {
    const int n = 128;
    Mat a(n, n, gls::CV_32FC1), b(n, n, gls::CV_32FC1), w(n, n, gls::CV_32FC1);
    std::mt19937 rng(3);
    std::uniform_real_distribution<float> u(0.f, 1.f);
    for (size_t i = 0; i < a.total(); i++) a.ptr<float>()[i] = u(rng);
    const int dx = 9, dy = -5;  // b = a shifted by (dx, dy), circularly
    for (int y = 0; y < n; y++)
        for (int x = 0; x < n; x++)
            b.ptr<float>(((y + dy) % n + n) % n)[((x + dx) % n + n) % n] = a.ptr<float>(y)[x];
    const double pi = 3.14159265358979323846;
    for (int y = 0; y < n; y++)
        for (int x = 0; x < n; x++)
            w.ptr<float>(y)[x] = (float)(0.25 * (1 - std::cos(2 * pi * y / (n - 1))) * (1 - std::cos(2 * pi * x / (n - 1))));
    GlsMat ga(a), gb(b), gw(w), none;
    double resp = 0;
    gls::Point2d s = gls::phaseCorrelate(ga, gb, gw, &resp);
    EXPECT(std::fabs(s.x - dx) < 0.05 && std::fabs(s.y - dy) < 0.05, "phaseCorrelate shift");
    EXPECT(resp > 0.3 && resp < 1.5, "phaseCorrelate response");
    gls::Point2d s2 = gls::phaseCorrelate(ga, gb, none);
    EXPECT(std::fabs(s2.x - dx) < 0.05 && std::fabs(s2.y - dy) < 0.05, "phaseCorrelate, no window");
    Mat a2 = ga;
    EXPECT(a2.ptr<float>()[17] == a.ptr<float>()[17], "inputs left unchanged");
    // the reference-arithmetic extension finds the same shift
    for (int algo = 0; algo < 2; algo++) {
        double rresp = 0;
        gls::Point2d r = gls::phaseCorrelateReference(ga, gb, gw, &rresp, algo);
        EXPECT(std::fabs(r.x - s.x) < 1e-3 && std::fabs(r.y - s.y) < 1e-3,
               "phaseCorrelateReference agrees with phaseCorrelate");
        EXPECT(std::fabs(rresp - resp) < 1e-4, "phaseCorrelateReference response");
    }
}

static void test_fft_reference() {
    const int rows = 32, cols = 64;
    Mat a(rows, cols, gls::CV_32FC2);
    std::mt19937 rng(11);
    std::uniform_real_distribution<float> u(-1.f, 1.f);
    for (size_t i = 0; i < 2 * a.total(); i++) a.ptr<float>()[i] = u(rng);
    GlsMat ga(a), fast, exact;
    gls::fft(ga, fast, gls::GLS_FFT_SHIFT);
    for (int algo = 0; algo < 2; algo++) {
        gls::fftReference(ga, exact, gls::GLS_FFT_SHIFT, algo);
        Mat f = fast, e = exact;
        double num = 0, den = 0;
        for (size_t i = 0; i < 2 * a.total(); i++) {
            const double d = (double)f.ptr<float>()[i] - e.ptr<float>()[i];
            num += d * d;
            den += (double)e.ptr<float>()[i] * e.ptr<float>()[i];
        }
        EXPECT(std::sqrt(num / den) < 1e-6, "fftReference agrees with fft within FP32 rounding");
    }
    // in place, as gls::fft allows
    GlsMat c = ga.clone();
    gls::fftReference(c, c, 0, 0);
    gls::fftReference(ga, exact, 0, 0);
    Mat cm = c, em = exact;
    bool same = true;
    for (size_t i = 0; i < 2 * a.total(); i++) same &= cm.ptr<float>()[i] == em.ptr<float>()[i];
    EXPECT(same, "fftReference in place equals out of place");
}

static void test_errors() {
    bool thrown = false;
    try {
        GlsMat g(Size(6, 8), gls::CV_32FC2), out;
        gls::fft(g, out);
    } catch (const gls::Exception &e) {
        thrown = e.status() == GLSFFT_ERROR_NOT_POW2;
    }
    EXPECT(thrown, "non power of two throws gls::Exception(NOT_POW2)");
    thrown = false;
    try {
        GlsMat a(Size(16, 16), gls::CV_32FC2), b(Size(16, 16), gls::CV_32FC2), w;
        gls::phaseCorrelate(a, b, w);
    } catch (const gls::Exception &) {
        thrown = true;
    }
    EXPECT(thrown, "phaseCorrelate on CV_32FC2 throws");
    thrown = false;
    try {
        GlsMat a(Size(16, 16), gls::CV_32FC1), b(Size(32, 16), gls::CV_32FC1), w;
        gls::phaseCorrelate(a, b, w);
    } catch (const gls::Exception &e) {
        thrown = e.status() == GLSFFT_ERROR_SHAPE;
    }
    EXPECT(thrown, "phaseCorrelate size mismatch throws");
}

// the spectrum operations, minMaxLoc and normalize, written like the
// reference's UnitTest_glsBasicOperation / UnitTest_glsMinMaxLoc checks
static void test_spectrum_ops() {
    const int R = 24, C = 32;  // the reference minMaxLoc test's size
    Mat a = random_complex(R, C, 31), b = random_complex(R, C, 32);
    GlsMat ga(a), gb(b), prod, conj_prod, poc, mag, lmag;
    gls::mulSpectrums(ga, gb, prod, false);
    gls::mulSpectrums(ga, gb, conj_prod, true);
    gls::mulSpectrumsPhaseOnly(ga, gb, poc);
    gls::magSpectrums(ga, mag);
    gls::logMagSpectrums(ga, lmag, 1.0f);
    Mat hp = prod, hc = conj_prod, hpoc = poc, hm = mag, hl = lmag;
    EXPECT(hm.type() == gls::CV_32FC1 && hl.type() == gls::CV_32FC1, "magnitudes are CV_32FC1");
    const float *pa = a.ptr<float>(), *pb = b.ptr<float>();
    double e_prod = 0, e_conj = 0, e_poc = 0, e_mag = 0, e_log = 0;
    for (size_t i = 0; i < a.total(); i++) {
        const std::complex<double> x(pa[2 * i], pa[2 * i + 1]), y(pb[2 * i], pb[2 * i + 1]);
        const std::complex<double> p = x * y, c = x * std::conj(y), n = c / std::abs(c);
        e_prod = std::fmax(e_prod, std::abs(p - std::complex<double>(hp.ptr<float>()[2 * i], hp.ptr<float>()[2 * i + 1])));
        e_conj = std::fmax(e_conj, std::abs(c - std::complex<double>(hc.ptr<float>()[2 * i], hc.ptr<float>()[2 * i + 1])));
        e_poc = std::fmax(e_poc, std::abs(n - std::complex<double>(hpoc.ptr<float>()[2 * i], hpoc.ptr<float>()[2 * i + 1])));
        e_mag = std::fmax(e_mag, std::fabs(std::abs(x) - hm.ptr<float>()[i]));
        e_log = std::fmax(e_log, std::fabs(std::log(std::abs(x) + 1.0) - hl.ptr<float>()[i]));
    }
    EXPECT(e_prod < 1e-6 && e_conj < 1e-6, "mulSpectrums matches a double product");
    EXPECT(e_poc < 1e-6, "mulSpectrumsPhaseOnly matches");
    EXPECT(e_mag < 1e-6 && e_log < 1e-6, "magSpectrums / logMagSpectrums match");

    Mat img(R, C, gls::CV_32FC1);
    std::mt19937 rng(33);
    std::uniform_real_distribution<float> u(-1.f, 1.f);
    float *pi = img.ptr<float>();
    for (size_t i = 0; i < img.total(); i++) pi[i] = u(rng);
    pi[5 * C + 7] = 3.f;   // maximum, once more later: the first one counts
    pi[20 * C + 1] = 3.f;
    pi[2 * C + 30] = -3.f;
    GlsMat gimg(img);
    double mn = 0, mx = 0;
    gls::Point lmin, lmax;
    gls::minMaxLoc(gimg, &mn, &mx, &lmin, &lmax);
    EXPECT(mn == -3.0 && mx == 3.0, "minMaxLoc values");
    EXPECT(lmin.x == 30 && lmin.y == 2 && lmax.x == 7 && lmax.y == 5, "minMaxLoc first occurrence");
    GlsMat nrm;
    gls::normalize(gimg, nrm, 0, 1, gls::NORM_MINMAX);
    Mat hn = nrm;
    EXPECT(hn.ptr<float>()[2 * C + 30] == 0.f && std::fabs(hn.ptr<float>()[5 * C + 7] - 1.f) < 1e-6f,
           "normalize NORM_MINMAX maps min to 0 and max to 1");
    // getDstMat: an output that aliases an input gets new storage, so other
    // copies of the input keep its data (glsMat.h:173-196)
    GlsMat a2(a), keep = a2;
    gls::mulSpectrums(a2, gb, a2, false);
    Mat hk = keep, ha2 = a2;
    EXPECT(!a2.shares(keep), "mulSpectrums into its own input gets new storage");
    EXPECT(hk.ptr<float>()[0] == a.ptr<float>()[0] && ha2.ptr<float>()[0] == hp.ptr<float>()[0],
           "the old copy keeps the input, the output has the product");
    // a CV_32FC1 image transformed into itself (dst is the same object as src)
    Mat r1(16, 16, gls::CV_32FC1);
    for (size_t i = 0; i < r1.total(); i++) r1.ptr<float>()[i] = (float)std::cos(0.11 * i);
    GlsMat self(r1), ref_out;
    gls::fft(self, ref_out);
    gls::fft(self, self);
    Mat hs = self, hr = ref_out;
    bool eq = self.type() == gls::CV_32FC2;
    for (size_t i = 0; i < 2 * hs.total(); i++) eq &= hs.ptr<float>()[i] == hr.ptr<float>()[i];
    EXPECT(eq, "fft(C, C) of a CV_32FC1 image");
    bool thrown = false;
    try {
        gls::normalize(gimg, nrm, 1, 0, gls::NORM_L2);
    } catch (const gls::Exception &) {
        thrown = true;
    }
    EXPECT(thrown, "normalize NORM_L2 is outside this path and throws");
}

int main() {
    gls::glsCvInit(0);
    test_fft();
    test_phase_correlate();
    test_fft_reference();
    test_errors();
    test_spectrum_ops();
    gls::glsCvTerminate();
    if (failures) {
        std::printf("%d FAILURES\n", failures);
        return 1;
    }
    std::printf("ALL OK\n");
    return 0;
}
