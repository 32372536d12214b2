"""Reference-arithmetic mode on the GPU: bit-identical to the reference.

glsfft_fft2d_reference runs the reference's own FP32 line arithmetic (the
radix-2 type1 Stockham of UnitTest_glsCV/fft_stockhum.cpp:436-538, or the
radix-4 Stockham of :866-1031 driven one line at a time, the GLSL shader's
algorithm) with the reference's twiddle table; the oracle restates the same
routines and is itself pinned bit for bit to the reference compiled from its
sources (tests/test_oracle.py).  So the GPU output must equal the oracle bit
for bit, for every flag combination, square and rectangular sizes, 1-D
lines, batches and in place.  glsfft_phase_correlate_reference composes the
reference's phaseCorrelate (glsPhaseCorrelate.cpp:142-236) on that FFT and
must give the oracle's dx, dy and response exactly.
"""
from __future__ import annotations

import numpy as np
import pytest

import glscv_gb300 as g
from glscv_gb300 import workloads as wl
from tests.gpu_util import stream_handle

pytestmark = pytest.mark.gpu

INV, SCALE, SHIFT = 1, 2, 64


@pytest.fixture()
def tctx(native, torch_cuda):
    c = g.Context(0)
    yield c
    c.close()


def _bits_equal(a, b):
    return np.array_equal(np.ascontiguousarray(a).view(np.uint32),
                          np.ascontiguousarray(b).view(np.uint32))


def _gpu(ctx, torch, x, flags, algo, inplace=False):
    rows, cols = x.shape
    d = torch.from_numpy(np.ascontiguousarray(x)).cuda()
    out = d if inplace else torch.empty_like(d)
    ctx.fft2d_reference(d.data_ptr(), out.data_ptr(), rows, cols, flags, algo, stream_handle(torch))
    torch.cuda.synchronize()
    return out.cpu().numpy()


@pytest.mark.parametrize("algo", [0, 1])
@pytest.mark.parametrize("shape", [(1, 1), (1, 64), (64, 1), (2, 2), (16, 16), (8, 32),
                                   (128, 256), (512, 512), (1024, 1024), (2048, 512)])
@pytest.mark.parametrize("flags", [0, INV | SCALE, SHIFT, INV | SHIFT])
def test_reference_fft_bit_exact(tctx, torch_cuda, oracle, algo, shape, flags):
    x = wl.complex_uniform(*shape, 1500 + shape[0] + 3 * shape[1] + flags)
    got = _gpu(tctx, torch_cuda, x, flags, algo)
    ref = oracle.fft2d(x, flags, algo)
    assert _bits_equal(got, ref)


@pytest.mark.parametrize("algo", [0, 1])
def test_reference_fft_4096_and_in_place(tctx, torch_cuda, oracle, algo):
    x = wl.complex_uniform(4096, 4096, 1531 + algo)
    ref = oracle.fft2d(x, INV | SCALE | SHIFT, algo)
    assert _bits_equal(_gpu(tctx, torch_cuda, x, INV | SCALE | SHIFT, algo, inplace=True), ref)


def test_reference_fft_batch(tctx, torch_cuda, oracle):
    torch = torch_cuda
    xs = np.stack([wl.complex_uniform(64, 128, 1540 + i) for i in range(5)])
    d = torch.from_numpy(xs).cuda()
    out = torch.empty_like(d)
    tctx.fft2d_reference(d.data_ptr(), out.data_ptr(), 64, 128, SHIFT, 1, stream_handle(torch), 5)
    torch.cuda.synchronize()
    got = out.cpu().numpy()
    for i in range(5):
        assert _bits_equal(got[i], oracle.fft2d(xs[i], SHIFT, 1))


def test_reference_mode_matches_fp64_like_the_default(tctx, torch_cuda, oracle):
    # the reference's radix-2 arithmetic is a correct FFT (error at the FP32
    # level of the default path)
    x = wl.complex_uniform(1024, 1024, 1550)
    y = _gpu(tctx, torch_cuda, x, 0, 0)
    assert oracle.rel_l2(y, oracle.fft2d_f64(x)) < 1e-6


@pytest.mark.parametrize("algo", [0, 1])
@pytest.mark.parametrize("shape,window", [((64, 64), True), ((256, 256), True), ((256, 256), False),
                                          ((512, 256), True), ((1024, 1024), True)])
def test_reference_phase_correlate_exact(tctx, torch_cuda, oracle, algo, shape, window):
    torch = torch_cuda
    rows, cols = shape
    a, b = wl.random_pair(rows, cols, seed=1560 + rows + cols, shift=(rows / 16 + 0.4, -cols / 32 - 0.3))
    w = wl.hann_window(rows, cols) if window else None
    (ox, oy), oresp, _, _ = oracle.phase_correlate(a, b, w, box=5, algo=algo, zero_guard=False)
    da = torch.from_numpy(np.ascontiguousarray(a, np.float32)).cuda()
    db = torch.from_numpy(np.ascontiguousarray(b, np.float32)).cuda()
    dw = torch.from_numpy(np.ascontiguousarray(w, np.float32)).cuda() if window else None
    (gx, gy), gresp = tctx.phase_correlate_reference(da.data_ptr(), db.data_ptr(),
                                                     dw.data_ptr() if window else None, rows, cols,
                                                     5, algo, stream_handle(torch))
    assert (gx, gy, gresp) == (ox, oy, oresp)


def test_reference_mode_rejects_bad_algo(tctx, torch_cuda):
    torch = torch_cuda
    d = torch.zeros(16, 16, dtype=torch.complex64, device="cuda")
    with pytest.raises(g.GlsError):
        tctx.fft2d_reference(d.data_ptr(), d.data_ptr(), 16, 16, 0, 2)


CONFIG_2B_SEEDS = [(6 + 100 * k, 7 + 100 * k) for k in range(8)]


@pytest.mark.parametrize("algo", [0, 1])
def test_reference_phase_correlate_zero_guard_config2b(tctx, torch_cuda, oracle, algo):
    """The benchmark phaseCorrelate configuration: 1024^2 smooth field
    (blurred noise, sigma 4 px), B = A rolled by an integer in [-100, 100]
    plus N(0, 0.01^2), Hann window, 8 seeds.  Its spectrum has bins where
    |F1 conj F2| is exactly 0 in FP32, so the reference's epsilon-free
    phase-only step returns NaN everywhere; with GLSFFT_REFERENCE_ZERO_GUARD
    those bins become 0 and the reference-arithmetic GPU path equals the
    oracle's guarded restatement bit for bit (dx, dy, response): 0 px."""
    torch = torch_cuda
    n = 1024
    w = wl.hann_window(n, n)
    dw = torch.from_numpy(w).cuda()
    for sf, ss in CONFIG_2B_SEEDS:
        a, b, (dx, dy) = wl.shifted_pair(n, n, seed_field=sf, seed_shift=ss, max_shift=100)
        (ox, oy), oresp, opeak, _ = oracle.phase_correlate(a, b, w, box=5, algo=algo,
                                                           zero_guard=True)
        da, db = torch.from_numpy(a).cuda(), torch.from_numpy(b).cuda()
        (gx, gy), gresp = tctx.phase_correlate_reference(
            da.data_ptr(), db.data_ptr(), dw.data_ptr(), n, n, 5,
            algo | g.REFERENCE_ZERO_GUARD, stream_handle(torch))
        assert (gx, gy, gresp) == (ox, oy, oresp), (sf, ss)
        assert opeak == ((n // 2 - int(dx)) % n, (n // 2 - int(dy)) % n)
