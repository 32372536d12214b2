"""Generate tests/golden/fft_golden.npz from the reference's own CPU Stockham.

Runs the reference code compiled from UnitTest_glsCV/fft_stockhum.cpp
(oracle/_ref/libref_stockham.so, built by oracle/build_ref.sh) on seeded
inputs mirroring the reference's FFT test cases (unittest_glsFft.cpp:203-422).
The reference routines are forward-only and unscaled; INVERSE, SCALE and SHIFT
are composed exactly as gls::fft defines them (conj in/out, x 1/rows x 1/cols,
quadrant swap).  Square cases use fft_dit_Stockham_radix2_type1
(fft_stockhum.cpp:436), 1-D and rectangular cases the radix-4 DIT routine
(fft_stockhum.cpp:771) one line at a time.

Usage (where the reference checkout and oracle/_ref exist):
    python tests/golden/make_golden.py
"""
from __future__ import annotations

import sys
from pathlib import Path

import numpy as np

ROOT = Path(__file__).resolve().parents[2]
sys.path.insert(0, str(ROOT))

from oracle import oracle as orc  # noqa: E402
from glscv_gb300.workloads import complex_uniform  # noqa: E402

# (name, rows, cols, flags, seed, algo) -- algo 0: radix-2 type1 square,
# 1: radix-4 lines.  Names follow the reference's TEST_METHODs.
CASES = [
    ("FFT_16x16", 16, 16, 0, 101, 0),
    ("FFT_32x32", 32, 32, 0, 102, 0),
    ("FFT_256x256", 256, 256, 0, 103, 0),
    ("FFT_32x32_SHFIT", 16, 16, orc.GLS_FFT_SHIFT, 104, 0),  # the reference test uses N=16
    ("FFT_128x128_SCALE", 128, 128, orc.DFT_SCALE, 105, 0),
    ("IFFT_64x64", 64, 64, orc.DFT_INVERSE, 106, 0),
    ("IFFT_32x32_SCALE", 32, 32, orc.DFT_INVERSE | orc.DFT_SCALE, 107, 0),
    ("FFT_32H", 1, 32, 0, 108, 1),
    ("FFT_64V", 64, 1, 0, 109, 1),
    ("FFT_64x128_RECT", 64, 128, 0, 110, 1),
    ("IFFT_128x32_RECT_SCALE_SHIFT", 128, 32,
     orc.DFT_INVERSE | orc.DFT_SCALE | orc.GLS_FFT_SHIFT, 111, 1),
]


def compose(x: np.ndarray, flags: int, algo: int) -> np.ndarray:
    rows, cols = x.shape
    inp = np.conj(x).astype(np.complex64) if flags & orc.DFT_INVERSE else x
    if algo == 0:
        y = orc.ref_fft_r2t1_square(inp)
    else:
        y = orc.ref_fft_r4_lines(inp)
    if flags & (orc.DFT_INVERSE | orc.DFT_SCALE):
        s = np.float32(1.0)
        if flags & orc.DFT_SCALE:
            s = np.float32(np.float32(1.0) / np.float32(rows)) * np.float32(np.float32(1.0) / np.float32(cols))
        sim = -s if flags & orc.DFT_INVERSE else s
        f = y.view(np.float32).reshape(rows, cols, 2).copy()
        f[..., 0] = f[..., 0] * s
        f[..., 1] = f[..., 1] * sim
        y = f.view(np.complex64).reshape(rows, cols)
    if flags & orc.GLS_FFT_SHIFT:
        y = np.roll(y, (rows // 2, cols // 2), axis=(0, 1))
    return np.ascontiguousarray(y)


def main() -> None:
    if orc.ref_lib() is None:
        orc.build_ref()
    if orc.ref_lib() is None:
        raise SystemExit("oracle/_ref is not built (reference checkout missing)")
    out = {}
    for name, rows, cols, flags, seed, algo in CASES:
        x = complex_uniform(rows, cols, seed)
        out[f"{name}__in"] = x
        out[f"{name}__out"] = compose(x, flags, algo)
        out[f"{name}__meta"] = np.array([rows, cols, flags, seed, algo], np.int64)
    path = Path(__file__).with_name("fft_golden.npz")
    np.savez_compressed(path, **out)
    print(f"wrote {path} ({path.stat().st_size} bytes, {len(CASES)} cases)")


if __name__ == "__main__":
    main()
