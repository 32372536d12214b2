"""gls::fft on the GPU through the C ABI, checked against the oracle.

The bar is the reference test's own (unittest_glsFft.cpp:101-105,
Unittest_Common.h:191): an element fails only if it is more than 64 ULPs AND
more than EPS = 1e-6 * N (1e-6 with SCALE) away from the reference result.
The reference result is the golden output of the reference's own CPU
Stockham where one exists, else the oracle; rel-L2 against an FP64 DFT is
checked too (<= 1e-6 at every size; FP32 Stockham reaches ~2-4e-7).
"""
from __future__ import annotations

import numpy as np
import pytest

from glscv_gb300 import workloads as wl
from tests.gpu_util import gpu_fft

pytestmark = pytest.mark.gpu

INV, SCALE, SHIFT = 1, 2, 64
ALL_FLAGS = [0, INV, SCALE, SHIFT, INV | SCALE, INV | SHIFT, SCALE | SHIFT, INV | SCALE | SHIFT]


def _check(oracle, ref, got, n, flags, x, tol_rel=1e-6):
    bad = oracle.are_equal(ref, got, 64, oracle.fft_eps(n, flags))
    assert bad == 0, f"{bad} components outside ULPS 64 / EPS {oracle.fft_eps(n, flags)}"
    err = oracle.rel_l2(got, oracle.fft2d_f64(x, flags))
    assert err < tol_rel, err


def test_reference_test_cases_against_golden(ctx, torch_cuda, oracle, golden):
    names = sorted({k.split("__")[0] for k in golden.files})
    for name in names:
        rows, cols, flags, seed, algo = (int(v) for v in golden[f"{name}__meta"])
        x = golden[f"{name}__in"]
        got = gpu_fft(ctx, torch_cuda, x, flags)
        _check(oracle, golden[f"{name}__out"], got, max(rows, cols), flags, x)


@pytest.mark.parametrize("n", [1, 2, 4, 8, 16, 32, 64, 128, 256, 512, 1024])
def test_square_sizes_vs_oracle(ctx, torch_cuda, oracle, n):
    x = wl.complex_uniform(n, n, 200 + n)
    for flags in (0, INV | SCALE):
        got = gpu_fft(ctx, torch_cuda, x, flags)
        _check(oracle, oracle.fft2d(x, flags), got, n, flags, x)


@pytest.mark.parametrize("n", [2048, 4096])
def test_large_square_vs_fp64(ctx, torch_cuda, oracle, n):
    """Unscaled: rel-L2 vs FP64.  The element-wise ULPS/EPS bar is applied with
    DFT_SCALE, as the reference's own 1024/2048 tests do
    (unittest_glsFft.cpp:348-385): unscaled at these sizes one of millions of
    components of two FP32 FFTs can differ by more than 1e-6*N."""
    x = wl.complex_uniform(n, n, 300 + n)
    got = gpu_fft(ctx, torch_cuda, x, 0)
    assert oracle.rel_l2(got, oracle.fft2d_f64(x)) < 1e-6
    got_s = gpu_fft(ctx, torch_cuda, x, SCALE)
    y = oracle.fft2d(x, SCALE, 1)  # the shader's radix-4 Stockham, line by line
    assert oracle.are_equal(y, got_s, 64, oracle.fft_eps(n, SCALE)) == 0


@pytest.mark.parametrize("shape", [(1, 32), (64, 1), (1, 4096), (4096, 1), (2, 8), (8, 2),
                                   (64, 128), (1024, 2048), (2048, 1024), (16, 4096),
                                   (4096, 16), (1, 1), (1, 2), (2, 1)])
def test_rect_and_1d_shapes(ctx, torch_cuda, oracle, shape):
    rows, cols = shape
    x = wl.complex_uniform(rows, cols, rows * 7 + cols)
    for flags in (0, INV | SCALE | SHIFT):
        got = gpu_fft(ctx, torch_cuda, x, flags)
        _check(oracle, oracle.fft2d(x, flags, 1), got, max(rows, cols), flags, x)


@pytest.mark.parametrize("flags", ALL_FLAGS)
def test_all_flag_combinations(ctx, torch_cuda, oracle, flags):
    x = wl.complex_uniform(64, 32, 11)
    got = gpu_fft(ctx, torch_cuda, x, flags)
    _check(oracle, oracle.fft2d(x, flags), got, 64, flags, x)


def test_inplace(ctx, torch_cuda, oracle):
    x = wl.complex_uniform(256, 256, 12)
    for flags in (0, INV | SHIFT):
        got = gpu_fft(ctx, torch_cuda, x, flags, inplace=True)
        _check(oracle, oracle.fft2d(x, flags), got, 256, flags, x)


@pytest.mark.parametrize("shape", [(32, 32), (1, 64), (64, 1), (256, 128)])
def test_real_input_promote(ctx, torch_cuda, oracle, shape):
    """CV_32FC1 input: gls::fft merges it to complex first (glsFft.cpp:684-689);
    imag = 0 here (the reference leaves the second plane's sampler unbound)."""
    rows, cols = shape
    r = np.random.default_rng(13).uniform(0, 1, shape).astype(np.float32)
    got = gpu_fft(ctx, torch_cuda, r, 0)
    xc = r.astype(np.complex64)
    _check(oracle, oracle.fft2d(xc, 0, 1), got, max(rows, cols), 0, xc)


def test_round_trip_256_config1(ctx, torch_cuda, oracle):
    """Forward then INVERSE|SCALE of one 256x256 uniform[-1,1] image, seed 0."""
    x = wl.complex_uniform(256, 256, 0)
    f = gpu_fft(ctx, torch_cuda, x, 0)
    y = gpu_fft(ctx, torch_cuda, f, INV | SCALE)
    assert oracle.rel_l2(f, oracle.fft2d_f64(x)) < 1e-6
    assert oracle.rel_l2(y, x) < 1e-6


def test_full_size_4096_properties(ctx, torch_cuda, oracle):
    """At 4096^2: Parseval, round trip and linearity (size-independent checks)."""
    n = 4096
    x = wl.complex_uniform(n, n, 2)
    f = gpu_fft(ctx, torch_cuda, x, 0)
    px = np.sum(np.abs(x.astype(np.complex128)) ** 2)
    pf = np.sum(np.abs(f.astype(np.complex128)) ** 2) / (n * n)
    assert abs(pf / px - 1) < 1e-6
    y = gpu_fft(ctx, torch_cuda, f, INV | SCALE)
    assert oracle.rel_l2(y, x) < 1e-6
    z = wl.complex_uniform(n, n, 3)
    fz = gpu_fft(ctx, torch_cuda, z, 0)
    fs = gpu_fft(ctx, torch_cuda, (x + 2 * z).astype(np.complex64), 0)
    assert oracle.rel_l2(fs, f.astype(np.complex128) + 2 * fz) < 1e-6


def test_dynamic_range_input(ctx, torch_cuda, oracle):
    x = wl.complex_dynamic_range(1024, 1024, 4)
    got = gpu_fft(ctx, torch_cuda, x, 0)
    assert oracle.rel_l2(got, oracle.fft2d_f64(x)) < 1e-6


def test_non_default_stream(ctx, torch_cuda, oracle):
    torch = torch_cuda
    s = torch.cuda.Stream()
    x = wl.complex_uniform(128, 128, 14)
    with torch.cuda.stream(s):
        got = gpu_fft(ctx, torch, x, 0)
    _check(oracle, oracle.fft2d(x, 0), got, 128, 0, x)


@pytest.mark.parametrize("shape,count,flags", [((64, 64), 5, 0), ((1024, 1024), 6, INV | SCALE),
                                               ((32, 128), 7, SHIFT), ((1, 256), 3, INV),
                                               ((512, 1), 2, SCALE)])
def test_batched_matches_single_image_path(ctx, torch_cuda, oracle, shape, count, flags):
    """glsfft_fft2d_batched and the batched pass entry points give, image by
    image, exactly what the single-image call gives (same kernels)."""
    torch = torch_cuda
    rows, cols = shape
    xs = np.stack([wl.complex_uniform(rows, cols, 500 + i) for i in range(count)])
    d = torch.from_numpy(xs).cuda()
    out = torch.empty_like(d)
    s = torch.cuda.current_stream().cuda_stream
    ctx.fft2d_batched(d.data_ptr(), out.data_ptr(), count, rows, cols, flags, s)
    out2 = torch.empty_like(d)
    ctx.fft_rows(d.data_ptr(), out2.data_ptr(), rows, cols, flags, s, count=count)
    ctx.fft_cols(out2.data_ptr(), out2.data_ptr(), rows, cols, flags, s, count=count)
    torch.cuda.synchronize()
    got, got2 = out.cpu().numpy(), out2.cpu().numpy()
    for i in range(count):
        single = gpu_fft(ctx, torch, xs[i], flags)
        assert np.array_equal(got[i].view(np.uint32), single.view(np.uint32)), i
        if rows > 1 and cols > 1:
            # fft_rows/fft_cols with INVERSE conjugate per pass: same values
            assert oracle.rel_l2(got2[i], single) < 1e-6
    _check(oracle, oracle.fft2d(xs[-1], flags, 1), got[-1], max(rows, cols), flags, xs[-1])


def test_errors_on_device(ctx, torch_cuda):
    import glscv_gb300 as g
    torch = torch_cuda
    d = torch.zeros((8, 8), dtype=torch.complex64, device="cuda")
    with pytest.raises(g.GlsError) as e:
        ctx.fft2d(d.data_ptr(), d.data_ptr(), 8, 6, 0)
    assert e.value.status == 2
    with pytest.raises(g.GlsError) as e:
        ctx.fft2d(d.data_ptr(), d.data_ptr(), 8, 8, 8)
    assert e.value.status == 1
