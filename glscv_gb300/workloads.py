"""Seeded synthetic inputs with the shapes and value distributions of the
benchmark configurations of this path (there is no public dataset: the
reference's own tests draw uniform random images, unittest_glsFft.cpp:127 and
UnitTest_glsPhaseCorrelate.cpp:87).  All generators are numpy PCG64
(``np.random.default_rng(seed)``) so inputs are identical on every machine.
"""
from __future__ import annotations

import numpy as np

SIZE_CLASSES = [(128, 128), (256, 256), (512, 512), (1024, 1024), (1024, 2048)]  # (rows, cols)
SIZE_WEIGHTS = [0.3, 0.3, 0.2, 0.15, 0.05]


def complex_uniform(rows: int, cols: int, seed: int) -> np.ndarray:
    """CV_32FC2 image, re and im i.i.d. uniform[-1, 1)."""
    rng = np.random.default_rng(seed)
    re = rng.uniform(-1.0, 1.0, (rows, cols))
    im = rng.uniform(-1.0, 1.0, (rows, cols))
    return (re + 1j * im).astype(np.complex64)


def complex_dynamic_range(rows: int, cols: int, seed: int) -> np.ndarray:
    """Magnitudes log-uniform in [1e-3, 1], phases uniform [0, 2 pi)."""
    rng = np.random.default_rng(seed)
    mag = 10.0 ** rng.uniform(-3.0, 0.0, (rows, cols))
    ph = rng.uniform(0.0, 2 * np.pi, (rows, cols))
    return (mag * np.exp(1j * ph)).astype(np.complex64)


def hann_window(rows: int, cols: int) -> np.ndarray:
    """Separable Hann window 0.5 (1 - cos(2 pi i / (n - 1))), the form
    cv::createHanningWindow builds (UnitTest_glsPhaseCorrelate.cpp:97)."""
    def w(n):
        if n == 1:
            return np.ones(1)
        i = np.arange(n, dtype=np.float64)
        return 0.5 * (1.0 - np.cos(2.0 * np.pi * i / (n - 1)))
    return np.outer(w(rows), w(cols)).astype(np.float32)


def smooth_field(rows: int, cols: int, seed: int, sigma: float = 4.0) -> np.ndarray:
    """White noise N(0,1), circularly Gaussian-blurred (sigma px), min-max
    scaled to [0, 1]; float32."""
    rng = np.random.default_rng(seed)
    noise = rng.standard_normal((rows, cols))
    fy = np.fft.fftfreq(rows)[:, None]
    fx = np.fft.fftfreq(cols)[None, :]
    g = np.exp(-2.0 * (np.pi * sigma) ** 2 * (fx ** 2 + fy ** 2))
    f = np.real(np.fft.ifft2(np.fft.fft2(noise) * g))
    f = (f - f.min()) / (f.max() - f.min())
    return f.astype(np.float32)


def shifted_pair(rows: int, cols: int, seed_field: int = 6, seed_shift: int = 7,
                 max_shift: int = 100, noise_sigma: float = 0.01,
                 subpixel: tuple[float, float] | None = None):
    """A = smooth_field; B = A circularly shifted by an integer (dx, dy) drawn
    from [-max_shift, max_shift] (+ an optional sub-pixel part applied with the
    Fourier shift theorem in FP64), plus N(0, noise_sigma^2).  Returns
    (A, B, (dx, dy)) with the total shift of B relative to A."""
    a = smooth_field(rows, cols, seed_field)
    rng = np.random.default_rng(seed_shift)
    lim_x = min(max_shift, cols // 2 - 1) if cols > 2 else 0
    lim_y = min(max_shift, rows // 2 - 1) if rows > 2 else 0
    dx = int(rng.integers(-lim_x, lim_x + 1)) if lim_x > 0 else 0
    dy = int(rng.integers(-lim_y, lim_y + 1)) if lim_y > 0 else 0
    b = np.roll(a.astype(np.float64), (dy, dx), axis=(0, 1))
    sx = sy = 0.0
    if subpixel is not None:
        sx, sy = subpixel
        fy = np.fft.fftfreq(rows)[:, None]
        fx = np.fft.fftfreq(cols)[None, :]
        b = np.real(np.fft.ifft2(np.fft.fft2(b) * np.exp(-2j * np.pi * (fx * sx + fy * sy))))
    b = b + rng.normal(0.0, noise_sigma, (rows, cols))
    return a, b.astype(np.float32), (dx + sx, dy + sy)


def random_pair(rows: int, cols: int, seed: int, shift: tuple[float, float],
                noise_sigma: float = 0.0):
    """The reference test's input distribution (UnitTest_glsPhaseCorrelate.cpp:
    45-97): a uniform [0, 1) image and a shifted copy.  Integer shifts are
    circular; a fractional part is applied with the Fourier shift theorem in
    FP64 (cv::warpAffine is not available).  Returns (A, B)."""
    rng = np.random.default_rng(seed)
    a = rng.uniform(0.0, 1.0, (rows, cols))
    sx, sy = shift
    fy = np.fft.fftfreq(rows)[:, None]
    fx = np.fft.fftfreq(cols)[None, :]
    b = np.real(np.fft.ifft2(np.fft.fft2(a) * np.exp(-2j * np.pi * (fx * sx + fy * sy))))
    if noise_sigma:
        b = b + rng.normal(0.0, noise_sigma, (rows, cols))
    return a.astype(np.float32), b.astype(np.float32)


def batch_sizes(n_images: int = 512, seed: int = 3):
    """(rows, cols) per image drawn from SIZE_CLASSES with SIZE_WEIGHTS."""
    rng = np.random.default_rng(seed)
    idx = rng.choice(len(SIZE_CLASSES), size=n_images, p=SIZE_WEIGHTS)
    return [SIZE_CLASSES[i] for i in idx]


def fft_flops(rows: int, cols: int) -> float:
    """5 N log2 N reporting convention, N = rows * cols."""
    n = rows * cols
    return 5.0 * n * np.log2(n) if n > 1 else 0.0


def fft_bytes(rows: int, cols: int) -> int:
    """Algorithmic HBM bytes of one 2-D complex FFT: one read and one write
    of 8-byte pixels per dimension."""
    return 32 * rows * cols
