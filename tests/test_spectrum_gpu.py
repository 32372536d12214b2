"""Spectrum operations, minMaxLoc, normalize(NORM_MINMAX) and glsCam's FFT
display pipeline on the GPU against the oracle's restatements of the
reference shaders (glsBasicOperation.cpp:92-212, glsMinMaxLoc.cpp:65-119,
glsNormalize.cpp:52-68, glsCam.cpp:196-203).  Element results are bit-exact
where the formula is products, sums, quotients and square roots; log()
results agree within 2 ulp (CUDA's logf is not correctly rounded)."""
from __future__ import annotations

import numpy as np
import pytest

import glscv_gb300 as g
from glscv_gb300 import workloads as wl
from tests.gpu_util import stream_handle

pytestmark = pytest.mark.gpu


def _c(rows, cols, seed):
    return wl.complex_uniform(rows, cols, seed)


def _dev(torch, x):
    return torch.from_numpy(np.ascontiguousarray(x)).cuda()


def _eq(a, b):
    return np.array_equal(np.asarray(a).view(np.uint32), np.asarray(b).view(np.uint32))


@pytest.mark.parametrize("shape", [(1, 1), (37, 53), (512, 512), (1024, 2048)])
def test_mul_spectrums_bit_exact(ctx, torch_cuda, oracle, shape):
    torch = torch_cuda
    a, b = _c(*shape, 10), _c(*shape, 11)
    da, db = _dev(torch, a), _dev(torch, b)
    s = stream_handle(torch)
    for conj in (False, True):
        d = torch.empty_like(da)
        ctx.mul_spectrums(da.data_ptr(), db.data_ptr(), d.data_ptr(), *shape, conj, s)
        torch.cuda.synchronize()
        assert _eq(d.cpu().numpy(), oracle.mul_spectrums(a, b, conj)), conj
    # in place into src0
    ctx.mul_spectrums(da.data_ptr(), db.data_ptr(), da.data_ptr(), *shape, True, s)
    torch.cuda.synchronize()
    assert _eq(da.cpu().numpy(), oracle.mul_spectrums(a, b, True))


@pytest.mark.parametrize("shape", [(7, 9), (1024, 1024)])
def test_phase_only_bit_exact_with_nan_on_zero(ctx, torch_cuda, oracle, shape):
    torch = torch_cuda
    a, b = _c(*shape, 12), _c(*shape, 13)
    a[0, 0] = 0  # t = 0 there: 0/0 = NaN, as the shader
    da, db = _dev(torch, a), _dev(torch, b)
    d = torch.empty_like(da)
    ctx.mul_spectrums_phase_only(da.data_ptr(), db.data_ptr(), d.data_ptr(), *shape,
                                 stream_handle(torch))
    torch.cuda.synchronize()
    got, ref = d.cpu().numpy(), oracle.mul_spectrums_phase_only(a, b)
    assert np.isnan(got[0, 0].real) and np.isnan(got[0, 0].imag)
    ok = ~np.isnan(ref.view(np.float32))
    assert np.array_equal(ok, ~np.isnan(got.view(np.float32)))
    assert _eq(got.view(np.float32)[ok], ref.view(np.float32)[ok])


@pytest.mark.parametrize("shape", [(1, 1), (33, 65), (2048, 2048)])
def test_mag_and_log_mag(ctx, torch_cuda, oracle, shape):
    torch = torch_cuda
    a = _c(*shape, 14) * np.float32(3)
    da = _dev(torch, a)
    d = torch.empty(shape, dtype=torch.float32, device="cuda")
    s = stream_handle(torch)
    ctx.mag_spectrums(da.data_ptr(), d.data_ptr(), *shape, s)
    torch.cuda.synchronize()
    assert _eq(d.cpu().numpy(), oracle.mag_spectrums(a))
    for off in (1.0, 0.0, -0.5):
        ctx.log_mag_spectrums(da.data_ptr(), d.data_ptr(), *shape, off, s)
        torch.cuda.synchronize()
        got, ref = d.cpu().numpy(), oracle.mag_spectrums(a, True, off)
        fin = np.isfinite(ref)
        assert np.array_equal(fin, np.isfinite(got))
        assert oracle.ulps(got[fin], ref[fin]).max() <= 2, off


def test_mag_output_may_not_overlap_input(ctx, torch_cuda):
    torch = torch_cuda
    da = _dev(torch, _c(16, 16, 15))
    with pytest.raises(g.GlsError) as e:
        ctx.mag_spectrums(da.data_ptr(), da.data_ptr(), 16, 16)
    assert e.value.status == 1


def _mm_cases():
    rng = np.random.default_rng(20)
    u = rng.uniform(-1, 1, (24, 32)).astype(np.float32)        # the reference test's size
    ties = np.zeros((64, 64), np.float32)
    ties[5, 7] = ties[40, 2] = ties[5, 9] = 9.0                 # max ties: first is (7, 5)
    ties[3, 60] = ties[3, 61] = ties[63, 0] = -9.0              # min ties: first is (60, 3)
    nan = u.copy()
    nan[0, :4] = np.nan
    inf = u.copy()
    inf[10, 10], inf[20, 20] = np.inf, -np.inf
    zeros = np.array([[0.0, -0.0], [-0.0, 0.0]], np.float32)
    lit = np.full((3, 5), np.float32(3.4028233e38))            # beyond the shader's literal
    big = rng.standard_normal((4096, 4096)).astype(np.float32)
    # large inputs: ties far apart (scanned by different blocks), and a size
    # that is not a multiple of the blocks' stride
    staged = np.zeros((2048, 2048), np.float32)
    staged[3, 100] = staged[1500, 5] = staged[2047, 2047] = 7.0   # max: first is (100, 3)
    staged[1000, 1000] = staged[10, 10] = -3.0                     # min: first is (10, 10)
    staged[0, 0] = np.nan
    tail = rng.uniform(-1, 1, (1500, 1500)).astype(np.float32)
    tail[1499, 1000] = tail[1499, 1499] = 50.0                     # max: first is (1000, 1499)
    tail[1499, 1200] = -50.0
    return [u, ties, nan, inf, zeros, lit, np.array([[2.5]], np.float32), big, staged, tail]


@pytest.mark.parametrize("case", range(10))
def test_min_max_loc_first_occurrence(ctx, torch_cuda, oracle, case):
    torch = torch_cuda
    x = _mm_cases()[case]
    d = _dev(torch, x)
    got = ctx.min_max_loc(d.data_ptr(), *x.shape, stream_handle(torch))
    ref = oracle.min_max_loc(x)
    assert got == ref


@pytest.mark.parametrize("shape", [(24, 32), (1000, 3), (2048, 2048)])
def test_normalize_minmax_bit_exact(ctx, torch_cuda, oracle, shape):
    torch = torch_cuda
    x = (np.random.default_rng(21).standard_normal(shape) * 7 + 2).astype(np.float32)
    d = _dev(torch, x)
    out = torch.empty_like(d)
    s = stream_handle(torch)
    for alpha, beta in ((0.0, 1.0), (-3.0, 255.0)):
        ctx.normalize_minmax(d.data_ptr(), out.data_ptr(), *shape, alpha, beta, s)
        torch.cuda.synchronize()
        assert _eq(out.cpu().numpy(), oracle.normalize_minmax(x, alpha, beta)), (alpha, beta)
    ctx.normalize_minmax(d.data_ptr(), d.data_ptr(), *shape, 0.0, 1.0, s)  # in place
    torch.cuda.synchronize()
    assert _eq(d.cpu().numpy(), oracle.normalize_minmax(x, 0.0, 1.0))


@pytest.mark.parametrize("shape,window", [((256, 256), True), ((1024, 1024), True),
                                          ((512, 128), False), ((1, 64), True)])
def test_fft_display_pipeline(ctx, torch_cuda, oracle, shape, window):
    torch = torch_cuda
    rows, cols = shape
    frame = wl.smooth_field(rows, cols, seed=22) if rows > 1 else \
        np.random.default_rng(22).uniform(0, 1, shape).astype(np.float32)
    win = wl.hann_window(rows, cols) if window else None
    df, dw = _dev(torch, frame), (_dev(torch, win) if window else None)
    out = torch.empty(shape, dtype=torch.float32, device="cuda")
    ctx.fft_display(df.data_ptr(), dw.data_ptr() if window else None, out.data_ptr(), rows, cols,
                    1.0, stream_handle(torch))
    torch.cuda.synchronize()
    got = out.cpu().numpy()
    ref = oracle.fft_display(frame, win, 1.0)
    assert got.min() == 0.0 and abs(float(got.max()) - 1.0) < 1e-6
    # the same pipeline in FP64: bins far below the DC term carry FP32
    # rounding noise that differs between FFT implementations, so the GPU
    # result must be as close to FP64 as the reference algorithm's FP32 is
    f = frame.astype(np.float64) * (win.astype(np.float64) if window else 1.0)
    lm = np.log(np.abs(np.fft.fftshift(np.fft.fft2(f))) + 1.0)
    ref64 = (lm - lm.min()) / (lm.max() - lm.min())
    e_gpu, e_ref = np.abs(got - ref64).max(), np.abs(ref - ref64).max()
    assert e_gpu <= 2 * e_ref + 1e-6, (e_gpu, e_ref)
    assert e_gpu < 1e-3
    # the brightest bin is the DC term, at the centre after the shift
    if rows > 1:
        assert np.unravel_index(np.argmax(got), got.shape) == (rows // 2, cols // 2)


def test_fft_display_4096_equals_composed_ops(ctx, torch_cuda):
    # 4096-point columns run the streamed column pass with the log-magnitude
    # epilogue; the fused pipeline must equal the same steps as separate
    # calls bit for bit: window * frame, gls::fft(SHIFT) of the promoted
    # product, logMagSpectrums(1), normalize(0, 1, NORM_MINMAX)
    torch = torch_cuda
    s = stream_handle(torch)
    n = 4096
    frame = wl.smooth_field(n, n, seed=23)
    win = wl.hann_window(n, n)
    df, dw = _dev(torch, frame), _dev(torch, win)
    fused = torch.empty((n, n), dtype=torch.float32, device="cuda")
    ctx.fft_display(df.data_ptr(), dw.data_ptr(), fused.data_ptr(), n, n, 1.0, s)
    prod = _dev(torch, (frame * win).astype(np.float32))
    spec = torch.empty((n, n), dtype=torch.complex64, device="cuda")
    ctx.fft2d(prod.data_ptr(), spec.data_ptr(), n, n, 64, s, real_input=True)
    lm = torch.empty((n, n), dtype=torch.float32, device="cuda")
    ctx.log_mag_spectrums(spec.data_ptr(), lm.data_ptr(), n, n, 1.0, s)
    composed = torch.empty_like(lm)
    ctx.normalize_minmax(lm.data_ptr(), composed.data_ptr(), n, n, 0.0, 1.0, s)
    torch.cuda.synchronize()
    assert _eq(fused.cpu().numpy(), composed.cpu().numpy())
    assert ctx.device_status() == 0


@pytest.mark.parametrize("n", [256, 1024, 4096])
def test_fft_display_back_to_back_frames(ctx, torch_cuda, n):
    # frames queued on one stream share the context's spectrum buffer and
    # min / max keys, and each call's three launches are chained by
    # programmatic dependent launch: every output must equal the same frame
    # displayed alone, bit for bit
    torch = torch_cuda
    s = stream_handle(torch)
    win = _dev(torch, wl.hann_window(n, n))
    frames = [_dev(torch, wl.smooth_field(n, n, seed=300 + i)) for i in range(3 if n == 4096 else 6)]
    outs = [torch.empty((n, n), dtype=torch.float32, device="cuda") for _ in frames]
    for f, o in zip(frames, outs):
        ctx.fft_display(f.data_ptr(), win.data_ptr(), o.data_ptr(), n, n, 1.0, s)
    torch.cuda.synchronize()
    got = [o.cpu().numpy() for o in outs]
    alone = torch.empty((n, n), dtype=torch.float32, device="cuda")
    for f, g_ in zip(frames, got):
        ctx.fft_display(f.data_ptr(), win.data_ptr(), alone.data_ptr(), n, n, 1.0, s)
        torch.cuda.synchronize()
        assert _eq(g_, alone.cpu().numpy())
