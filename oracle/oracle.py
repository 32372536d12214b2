"""CPU oracle for the glsCV FFT / phaseCorrelate path.

TEST INFRASTRUCTURE ONLY: imported by tests/, ``__graft_entry__.smoke()`` and
the CPU-baseline leg of ``bench.py`` as the checker and the timed CPU baseline.
The product library (``glscv_gb300``) never imports or calls anything here.

* ``liboracle.so`` (built from ``oracle/stockham.c``) restates the reference's
  FP32 Stockham FFT (UnitTest_glsCV/fft_stockhum.cpp:436-538 and :771-1033)
  and gls::phaseCorrelate (glsCV/glsPhaseCorrelate.cpp:142-231).
* ``oracle/_ref/libref_stockham.so`` (built by ``oracle/build_ref.sh`` where
  the reference checkout exists) is the reference's own fft_stockhum.cpp;
  it pins the restatement bit for bit.
* FP64 references: numpy complex128 FFTs, the error yardstick for every size.
"""
from __future__ import annotations

import ctypes
import os
import subprocess
from pathlib import Path

import numpy as np

HERE = Path(__file__).resolve().parent
LIB_PATH = HERE / "liboracle.so"
REF_LIB_PATH = HERE / "_ref" / "libref_stockham.so"

DFT_INVERSE = 1
DFT_SCALE = 2
GLS_FFT_SHIFT = 64

_f32p = ctypes.POINTER(ctypes.c_float)
_dp = ctypes.POINTER(ctypes.c_double)
_ip = ctypes.POINTER(ctypes.c_int)

_lib = None
_ref = None


def build(force: bool = False) -> Path:
    """Compile oracle/stockham.c into oracle/liboracle.so (gcc, OpenMP)."""
    src = HERE / "stockham.c"
    if force or not LIB_PATH.exists() or LIB_PATH.stat().st_mtime < src.stat().st_mtime:
        tmp = LIB_PATH.with_suffix(".so.tmp")
        subprocess.check_call([
            "gcc", "-std=c11", "-O2", "-fPIC", "-fopenmp", "-ffp-contract=off", "-shared",
            "-o", str(tmp), str(src), "-lm"])
        os.replace(tmp, LIB_PATH)
    return LIB_PATH


REFERENCE_ENV = "GLS_REFERENCE_ROOT"


def reference_root() -> str | None:
    """The glsCV checkout named by the GLS_REFERENCE_ROOT environment
    variable, or None when it is unset or holds no fft_stockhum.cpp."""
    root = os.environ.get(REFERENCE_ENV)
    if root and Path(root, "UnitTest_glsCV", "fft_stockhum.cpp").exists():
        return root
    return None


def build_ref(reference_root_dir: str | None = None) -> Path | None:
    """Build oracle/_ref from a glsCV checkout (the argument, else
    GLS_REFERENCE_ROOT) when one is present; None otherwise."""
    script = HERE / "build_ref.sh"
    root = reference_root_dir or reference_root()
    if not root or not Path(root, "UnitTest_glsCV", "fft_stockhum.cpp").exists():
        return None
    subprocess.check_call(["bash", str(script), root],
                          stdout=subprocess.DEVNULL)
    return REF_LIB_PATH


def lib():
    global _lib
    if _lib is None:
        if not LIB_PATH.exists():
            build()
        l = ctypes.CDLL(str(LIB_PATH))
        l.oracle_fft_r2t1_square.argtypes = [_f32p, _f32p, ctypes.c_int]
        l.oracle_fft2d.argtypes = [_f32p, _f32p, ctypes.c_int, ctypes.c_int, ctypes.c_int,
                                   ctypes.c_int]
        l.oracle_phase_correlate.argtypes = [
            _f32p, _f32p, _f32p, ctypes.c_int, ctypes.c_int, ctypes.c_int, ctypes.c_int,
            ctypes.c_int, _dp, _dp, _dp, _f32p, _ip]
        l.oracle_max_loc.argtypes = [_f32p, ctypes.c_int, ctypes.c_int, _ip, _ip, _f32p]
        l.oracle_centroid.argtypes = [_f32p, ctypes.c_int, ctypes.c_int, ctypes.c_int,
                                      ctypes.POINTER(ctypes.c_double),
                                      ctypes.POINTER(ctypes.c_double),
                                      ctypes.POINTER(ctypes.c_double), _ip]
        l.oracle_centroid.restype = None
        l.oracle_mul_spectrums.argtypes = [_f32p, _f32p, _f32p, ctypes.c_size_t, ctypes.c_int]
        l.oracle_mul_spectrums_poc.argtypes = [_f32p, _f32p, _f32p, ctypes.c_size_t]
        l.oracle_mag_spectrums.argtypes = [_f32p, _f32p, ctypes.c_size_t, ctypes.c_int,
                                           ctypes.c_float]
        l.oracle_min_max_loc.argtypes = [_f32p, ctypes.c_int, ctypes.c_int, _dp, _dp, _ip, _ip]
        l.oracle_normalize_minmax.argtypes = [_f32p, _f32p, ctypes.c_int, ctypes.c_int,
                                              ctypes.c_double, ctypes.c_double]
        l.oracle_set_threads.argtypes = [ctypes.c_int]
        _lib = l
    return _lib


def ref_lib():
    """The reference's own fft_stockhum.cpp, or None where it was not built."""
    global _ref
    if _ref is None and REF_LIB_PATH.exists():
        l = ctypes.CDLL(str(REF_LIB_PATH))
        l.ref_fft_r2t1_square.argtypes = [_f32p, _f32p, ctypes.c_int]
        l.ref_fft_dif_r4_square.argtypes = [_f32p, _f32p, ctypes.c_int]
        l.ref_fft_r4_lines.argtypes = [_f32p, _f32p, ctypes.c_int, ctypes.c_int]
        _ref = l
    return _ref


def _fp(a: np.ndarray):
    return a.ctypes.data_as(_f32p)


def _c64(x: np.ndarray) -> np.ndarray:
    return np.ascontiguousarray(x, dtype=np.complex64)


def set_threads(n: int) -> None:
    lib().oracle_set_threads(int(n))


def num_threads() -> int:
    return int(lib().oracle_num_threads())


def fft2d(x: np.ndarray, flags: int = 0, algo: int = 0) -> np.ndarray:
    """gls::fft semantics on a complex64 (rows, cols) image; algo 0 = radix-2
    type1 Stockham lines, 1 = radix-4 Stockham lines (the shader's)."""
    x = _c64(x)
    out = np.empty_like(x)
    rows, cols = x.shape
    rc = lib().oracle_fft2d(_fp(x.view(np.float32)), _fp(out.view(np.float32)), rows, cols,
                            int(flags), int(algo))
    if rc != 0:
        raise ValueError(f"oracle_fft2d failed ({rc}) for shape {x.shape}")
    return out


def fft_r2t1_square(x: np.ndarray) -> np.ndarray:
    x = _c64(x)
    out = np.empty_like(x)
    rc = lib().oracle_fft_r2t1_square(_fp(x.view(np.float32)), _fp(out.view(np.float32)),
                                      x.shape[0])
    if rc != 0:
        raise ValueError("oracle_fft_r2t1_square failed")
    return out


def ref_fft_r2t1_square(x: np.ndarray) -> np.ndarray:
    x = _c64(x)
    out = np.empty_like(x)
    if ref_lib().ref_fft_r2t1_square(_fp(x.view(np.float32)), _fp(out.view(np.float32)),
                                     x.shape[0]) != 0:
        raise ValueError("reference fft_dit_Stockham_radix2_type1 failed")
    return out


def ref_fft_r4_lines(x: np.ndarray) -> np.ndarray:
    x = _c64(x)
    out = np.empty_like(x)
    if ref_lib().ref_fft_r4_lines(_fp(x.view(np.float32)), _fp(out.view(np.float32)),
                                  x.shape[0], x.shape[1]) != 0:
        raise ValueError("reference fft_dit_Stockham_radix4_type0 failed")
    return out


def max_loc(c: np.ndarray):
    c = np.ascontiguousarray(c, dtype=np.float32)
    px, py = ctypes.c_int(), ctypes.c_int()
    mv = ctypes.c_float()
    lib().oracle_max_loc(_fp(c), c.shape[0], c.shape[1], ctypes.byref(px), ctypes.byref(py),
                         ctypes.byref(mv))
    return (px.value, py.value), mv.value


def centroid(surface: np.ndarray, box: int = 5):
    """The tail of gls::phaseCorrelate on a given surface: ((dx, dy), response, peak)."""
    c = np.ascontiguousarray(surface, dtype=np.float32)
    dx, dy, resp = ctypes.c_double(), ctypes.c_double(), ctypes.c_double()
    peak = (ctypes.c_int * 2)()
    lib().oracle_centroid(_fp(c), c.shape[0], c.shape[1], int(box), ctypes.byref(dx),
                          ctypes.byref(dy), ctypes.byref(resp), ctypes.cast(peak, _ip))
    return (dx.value, dy.value), resp.value, (peak[0], peak[1])


def phase_correlate(a: np.ndarray, b: np.ndarray, window: np.ndarray | None = None,
                    box: int = 5, algo: int = 0, want_surface: bool = False,
                    zero_guard: bool = True):
    """gls::phaseCorrelate restated; returns ((dx, dy), response, peak, surface).
    zero_guard=False reproduces the reference's 0/0 -> NaN phase-only step."""
    a = np.ascontiguousarray(a, dtype=np.float32)
    b = np.ascontiguousarray(b, dtype=np.float32)
    rows, cols = a.shape
    wp = None
    if window is not None:
        window = np.ascontiguousarray(window, dtype=np.float32)
        wp = _fp(window)
    dx, dy, resp = ctypes.c_double(), ctypes.c_double(), ctypes.c_double()
    surf = np.empty((rows, cols), np.float32) if want_surface else None
    peak = (ctypes.c_int * 2)()
    rc = lib().oracle_phase_correlate(_fp(a), _fp(b), wp, rows, cols, int(box), int(algo),
                                      int(bool(zero_guard)), ctypes.byref(dx), ctypes.byref(dy), ctypes.byref(resp),
                                      _fp(surf) if surf is not None else None,
                                      ctypes.cast(peak, _ip))
    if rc != 0:
        raise ValueError(f"oracle_phase_correlate failed ({rc})")
    return (dx.value, dy.value), resp.value, (peak[0], peak[1]), surf


def mul_spectrums(a: np.ndarray, b: np.ndarray, conj: bool = False) -> np.ndarray:
    a, b = _c64(a), _c64(b)
    out = np.empty_like(a)
    lib().oracle_mul_spectrums(_fp(a.view(np.float32)), _fp(b.view(np.float32)),
                               _fp(out.view(np.float32)), a.size, int(conj))
    return out


def mul_spectrums_phase_only(a: np.ndarray, b: np.ndarray) -> np.ndarray:
    a, b = _c64(a), _c64(b)
    out = np.empty_like(a)
    lib().oracle_mul_spectrums_poc(_fp(a.view(np.float32)), _fp(b.view(np.float32)),
                                   _fp(out.view(np.float32)), a.size)
    return out


def mag_spectrums(a: np.ndarray, log_mag: bool = False, offset: float = 0.0) -> np.ndarray:
    a = _c64(a)
    out = np.empty(a.shape, np.float32)
    lib().oracle_mag_spectrums(_fp(a.view(np.float32)), _fp(out), a.size, int(log_mag),
                               ctypes.c_float(offset))
    return out


def min_max_loc(x: np.ndarray):
    """((min, max), (min_x, min_y), (max_x, max_y)) with gls::minMaxLoc semantics."""
    x = np.ascontiguousarray(x, dtype=np.float32)
    mn, mx = ctypes.c_double(), ctypes.c_double()
    lmin, lmax = (ctypes.c_int * 2)(), (ctypes.c_int * 2)()
    lib().oracle_min_max_loc(_fp(x), x.shape[0], x.shape[1], ctypes.byref(mn), ctypes.byref(mx),
                             ctypes.cast(lmin, _ip), ctypes.cast(lmax, _ip))
    return (mn.value, mx.value), (lmin[0], lmin[1]), (lmax[0], lmax[1])


def normalize_minmax(x: np.ndarray, alpha: float = 0.0, beta: float = 1.0) -> np.ndarray:
    x = np.ascontiguousarray(x, dtype=np.float32)
    out = np.empty_like(x)
    lib().oracle_normalize_minmax(_fp(x), _fp(out), x.shape[0], x.shape[1],
                                  ctypes.c_double(alpha), ctypes.c_double(beta))
    return out


def fft_display(frame: np.ndarray, window: np.ndarray | None, offset: float = 1.0) -> np.ndarray:
    """glsCam's FFT view (glsCam/glsCam.cpp:196-203): window * frame, gls::fft
    with GLS_FFT_SHIFT, logMagSpectrums(offset), normalize(0, 1, NORM_MINMAX)."""
    f = np.ascontiguousarray(frame, dtype=np.float32)
    if window is not None:
        f = (np.ascontiguousarray(window, dtype=np.float32) * f).astype(np.float32)
    spec = fft2d(f.astype(np.complex64), GLS_FFT_SHIFT, 0)
    return normalize_minmax(mag_spectrums(spec, True, offset), 0.0, 1.0)


# ---------------------------------------------------------------- FP64 yardstick

def fft2d_f64(x: np.ndarray, flags: int = 0) -> np.ndarray:
    """gls::fft / cv::dft semantics in complex128 (numpy pocketfft)."""
    x = np.asarray(x, dtype=np.complex128)
    rows, cols = x.shape
    axes = tuple(ax for ax, n in ((0, rows), (1, cols)) if n > 1)
    if flags & DFT_INVERSE:
        y = np.fft.ifftn(x, axes=axes) * (rows * cols) if axes else x.copy()
    else:
        y = np.fft.fftn(x, axes=axes) if axes else x.copy()
    if flags & DFT_SCALE:
        y = y / (rows * cols)
    if flags & GLS_FFT_SHIFT:
        y = np.roll(y, (rows // 2, cols // 2), axis=(0, 1))
    return y


def rel_l2(y: np.ndarray, ref: np.ndarray) -> float:
    ref = np.asarray(ref, dtype=np.complex128)
    d = np.asarray(y, dtype=np.complex128) - ref
    den = np.linalg.norm(ref.ravel())
    return float(np.linalg.norm(d.ravel()) / (den if den > 0 else 1.0))


def max_abs(y: np.ndarray, ref: np.ndarray) -> float:
    return float(np.max(np.abs(np.asarray(y, np.complex128) - np.asarray(ref, np.complex128))))


def ulps(a: np.ndarray, b: np.ndarray) -> np.ndarray:
    """ULP distance of float32 values, as Unittest_Common.h:61-71 computes it."""
    ai = np.ascontiguousarray(a, np.float32).view(np.int32).astype(np.int64)
    bi = np.ascontiguousarray(b, np.float32).view(np.int32).astype(np.int64)
    ai = np.where(ai < 0, 0x80000000 - ai, ai)
    bi = np.where(bi < 0, 0x80000000 - bi, bi)
    return np.abs(ai - bi)


def are_equal(ref: np.ndarray, dst: np.ndarray, max_ulps: int = 64, max_diff: float = 1e-6):
    """AreEqual<float>(Mat, Mat, maxUlps, maxDiff), Unittest_Common.h:160-215:
    an element fails only if ulps > maxUlps AND |diff| > maxDiff.  Returns the
    number of failing float components."""
    r = np.ascontiguousarray(ref).view(np.float32).ravel()
    d = np.ascontiguousarray(dst).view(np.float32).ravel()
    bad = (ulps(r, d) > max_ulps) & (np.abs(r - d) > max_diff)
    return int(np.count_nonzero(bad))


def fft_eps(n: int, flags: int) -> float:
    """The reference FFT test tolerance (unittest_glsFft.cpp:101-105)."""
    eps = 1e-6
    if not (flags & DFT_SCALE):
        eps *= n
    return np.float32(eps).item()


def phase_correlate_f64(a: np.ndarray, b: np.ndarray, window: np.ndarray | None = None,
                        box: int = 5, zero_guard: bool = True, want_surface: bool = False):
    """gls::phaseCorrelate (glsCV/glsPhaseCorrelate.cpp:142-231) restated in
    FP64 / complex128 on the same float32 inputs: window product (exact in
    FP64), forward 2-D DFTs (numpy pocketfft), phase-only cross spectrum
    F1 conj(F2) / |F1 conj(F2)| (glsBasicOperation.cpp:195-206; with
    zero_guard a bin with |.| = 0 becomes 0 instead of 0/0), unscaled inverse
    with the quadrant shift (:199), real part (:202-204), first maximum in
    row-major order (glsMinMaxLoc.cpp:65-119), clamped-box weighted centroid
    with DBL_EPSILON (:60-137), shift = center - centroid and response =
    sum / (rows*cols) (:219-231).  Returns ((dx, dy), response, peak,
    surface or None); the surface is float64."""
    a64 = np.asarray(a, dtype=np.float32).astype(np.float64)
    b64 = np.asarray(b, dtype=np.float32).astype(np.float64)
    if window is not None:
        w64 = np.asarray(window, dtype=np.float32).astype(np.float64)
        a64, b64 = a64 * w64, b64 * w64
    rows, cols = a64.shape
    f1 = np.fft.fft2(a64)
    f2 = np.fft.fft2(b64)
    t = f1 * np.conj(f2)
    mag = np.abs(t)
    with np.errstate(invalid="ignore", divide="ignore"):
        p = t / mag
    if zero_guard:
        p[~(mag > 0)] = 0.0
    # unscaled inverse = rows*cols * ifft2, then the quadrant swap
    c = np.fft.ifft2(p) * (rows * cols)
    c = np.roll(c, (rows // 2, cols // 2), axis=(0, 1))
    re = np.ascontiguousarray(c.real)
    # first maximum in row-major order (NaN never wins)
    flat = np.where(np.isnan(re), -np.inf, re).ravel()
    idx = int(np.argmax(flat))
    py, px = divmod(idx, cols)
    h = box >> 1
    minr, maxr = max(py - h, 0), min(py + h, rows - 1)
    minc, maxc = max(px - h, 0), min(px + h, cols - 1)
    sx = sy = s = 0.0
    for y in range(minr, maxr + 1):
        for x in range(minc, maxc + 1):
            v = float(re[y, x])
            sx += x * v
            sy += y * v
            s += v
    response = s / (rows * cols)
    s += np.finfo(np.float64).eps
    dx = cols / 2.0 - sx / s
    dy = rows / 2.0 - sy / s
    return (dx, dy), response, (px, py), (re if want_surface else None)
