"""Pass schedules and the autotuner on the GPU.

Every selectable schedule of the row and column passes (radix bound,
elements per thread, lines / columns per block) must compute gls::fft within
the reference test's bar against the oracle (unittest_glsFft.cpp:101-105:
ULPS 64 / EPS 1e-6*N) and within FP32 error of an FP64 DFT.  The plain-path
autotuner and the batch-plan autotuner must pick an available schedule,
persist it in the plan cache and take it back from there untimed, and the
batch tuner must not touch the plan's own images.  Each test uses its own
context, so tuned schedules do not leak into other tests.
"""
from __future__ import annotations

import numpy as np
import pytest

import glscv_gb300 as g
from glscv_gb300 import workloads as wl
from tests.gpu_util import gpu_fft, stream_handle

pytestmark = pytest.mark.gpu

INV, SCALE, SHIFT = 1, 2, 64


@pytest.fixture()
def tctx(native, torch_cuda):
    c = g.Context(0)
    yield c
    c.close()


SHAPES = [(64, 64), (128, 256), (512, 512), (1024, 1024), (2048, 1024), (1024, 4096)]


@pytest.mark.parametrize("shape", SHAPES)
def test_every_schedule_matches_oracle(tctx, torch_cuda, oracle, shape):
    rows, cols = shape
    x = wl.complex_uniform(rows, cols, 900 + rows + cols)
    ref64 = oracle.fft2d_f64(x)
    small = max(rows, cols) <= 1024
    ref = oracle.fft2d(x, 0, 1) if small else None
    eps = oracle.fft_eps(max(rows, cols), 0) * 2
    pairs = [(r, 0) for r in range(7) if g.schedule_available(cols, r, False)]
    pairs += [(0, c) for c in range(1, 7) if g.schedule_available(rows, c, True)]
    assert len(pairs) >= 5
    for r, c in pairs:
        tctx.set_fft_schedule(rows, cols, r, c)
        assert tctx.get_fft_schedule(rows, cols) == (r, c)
        y = gpu_fft(tctx, torch_cuda, x, 0)
        assert oracle.rel_l2(y, ref64) < 5e-7, (r, c)
        if small:
            assert oracle.are_equal(ref, y, 64, eps) == 0, (r, c)
        # the inverse with scale brings the image back
        back = gpu_fft(tctx, torch_cuda, y, INV | SCALE)
        assert oracle.rel_l2(back, x) < 5e-7, (r, c)
    tctx.set_fft_schedule(rows, cols, 0, 0)
    assert tctx.get_fft_schedule(rows, cols) == (0, 0)


def test_schedule_flags_and_batched_path(tctx, torch_cuda, oracle):
    """Non-default schedules with INVERSE / SCALE / SHIFT through the batched
    entry point agree with the oracle."""
    torch = torch_cuda
    rows, cols = 256, 512
    xs = np.stack([wl.complex_uniform(rows, cols, 950 + i) for i in range(3)])
    d = torch.from_numpy(xs).cuda()
    o = torch.empty_like(d)
    for r, c in [(1, 1), (2, 2), (3, 4), (4, 3)]:
        tctx.set_fft_schedule(rows, cols, r, c)
        for flags in (SHIFT, INV | SCALE, INV | SHIFT):
            tctx.fft2d_batched(d.data_ptr(), o.data_ptr(), 3, rows, cols, flags,
                               stream_handle(torch))
            torch.cuda.synchronize()
            y = o.cpu().numpy()
            for i in range(3):
                ref = oracle.fft2d(xs[i], flags, 1)
                assert oracle.are_equal(ref, y[i], 64, oracle.fft_eps(cols, flags) * 2) == 0, \
                    (r, c, flags, i)


def test_unavailable_schedules_are_refused(tctx):
    with pytest.raises(g.GlsError):
        tctx.set_fft_schedule(16, 16, 1, 0)           # below the schedule minimum length
    with pytest.raises(g.GlsError):
        tctx.set_fft_schedule(4096, 4096, 0, 2)       # E=64 does not exist
    with pytest.raises(g.GlsError):
        tctx.set_fft_schedule(1024, 1024, 7, 0)
    with pytest.raises(g.GlsError):
        tctx.set_fft_schedule(1000, 1024, 0, 0)       # not a power of two


def test_autotune_fft2d_and_cache(tctx, torch_cuda, oracle, tmp_path):
    cache = str(tmp_path / "plans.jsonl")
    r1 = tctx.autotune_fft2d(1024, 1024, 8, cache, stream_handle(torch_cuda))
    assert not r1["from_cache"]
    assert g.schedule_available(1024, r1["row_schedule"], False)
    assert g.schedule_available(1024, r1["col_schedule"], True)
    assert 0 < r1["ms"] <= r1["ms_default"] * 1.0001
    assert tctx.get_fft_schedule(1024, 1024) == (r1["row_schedule"], r1["col_schedule"])
    # a fresh context takes the choice from the cache without timing
    with g.Context(0) as c2:
        r2 = c2.autotune_fft2d(1024, 1024, 8, cache, stream_handle(torch_cuda))
        assert r2["from_cache"]
        assert (r2["row_schedule"], r2["col_schedule"]) == (r1["row_schedule"], r1["col_schedule"])
        assert c2.get_fft_schedule(1024, 1024) == (r1["row_schedule"], r1["col_schedule"])
    # another count is another key
    r3 = tctx.autotune_fft2d(1024, 1024, 2, cache, stream_handle(torch_cuda))
    assert not r3["from_cache"]
    lines = open(cache).read().strip().splitlines()
    assert len(lines) == 2 and all('"kind": "fft2d"' in ln for ln in lines)
    # the tuned path still computes gls::fft
    x = wl.complex_uniform(1024, 1024, 961)
    y = gpu_fft(tctx, torch_cuda, x, 0)
    assert oracle.are_equal(oracle.fft2d(x, 0, 1), y, 64, oracle.fft_eps(1024, 0) * 2) == 0


def test_autotune_without_cache_path(tctx, torch_cuda):
    r = tctx.autotune_fft2d(256, 256, 4, None, stream_handle(torch_cuda))
    assert not r["from_cache"] and r["ms"] > 0


def _plan(ctx, torch, shapes, flags, inplace=False, seed0=980):
    xs = [wl.complex_uniform(r, c, seed0 + i) for i, (r, c) in enumerate(shapes)]
    d_in = [torch.from_numpy(x).cuda() for x in xs]
    d_out = d_in if inplace else [torch.zeros_like(d) for d in d_in]
    b = g.Batch(ctx, [d.data_ptr() for d in d_in], [d.data_ptr() for d in d_out], shapes, flags)
    return b, xs, d_in, d_out


def test_batch_autotune_leaves_images_untouched_and_caches(tctx, torch_cuda, oracle, tmp_path):
    torch = torch_cuda
    s = stream_handle(torch)
    cache = str(tmp_path / "plans.jsonl")
    shapes = [(256, 256), (1024, 1024), (128, 128), (512, 512), (2048, 2048), (1024, 2048)]
    b, xs, d_in, d_out = _plan(tctx, torch, shapes, (0, INV | SCALE))
    before_in = [d.cpu().numpy().copy() for d in d_in]
    res = b.autotune(cache, reps=3, stream=s)
    torch.cuda.synchronize()
    # the caller's buffers were neither read into nor written
    for i in range(len(shapes)):
        assert np.array_equal(d_in[i].cpu().numpy(), before_in[i])
        assert not d_out[i].cpu().numpy().any()
    assert not res["from_cache"]
    assert res["candidates"] == 3 * 6 * 7 + 6  # WS1-3: 6 lags x (3 chunks x 2 + deep); plain: 6
    assert res["variant"] in (0, 1, 2, 3) and 1 <= res["claim_chunk"] <= 4
    assert b.schedule()["variant"] == res["variant"]
    assert b.schedule()["lag_items"] == res["lag_items"]
    assert 0 < res["ms"] <= res["ms_default"] * 1.0001
    # the tuned plan computes the round trip
    b.execute(s)
    assert b.status(s) == 0
    for i, x in enumerate(xs):
        assert oracle.rel_l2(d_out[i].cpu().numpy(), x) < 5e-7, shapes[i]
    # the 2048 x 2048 image (own launches) follows the context's tuned schedule
    # bit for bit
    y = gpu_fft(tctx, torch, xs[4], 0)
    y = gpu_fft(tctx, torch, y, INV | SCALE)
    assert np.array_equal(d_out[4].cpu().numpy().view(np.uint32), y.view(np.uint32))
    # a second plan of the same shapes takes the schedule from the cache
    b2, _, _, _ = _plan(tctx, torch, shapes, (0, INV | SCALE), seed0=1200)
    res2 = b2.autotune(cache, reps=3, stream=s)
    assert res2["from_cache"]
    for k in ("variant", "claim_chunk", "claim_ahead", "lag_items"):
        assert res2[k] == res[k], k
    b.close()
    b2.close()


def test_batch_autotune_inplace_plan_untouched(tctx, torch_cuda, oracle):
    torch = torch_cuda
    s = stream_handle(torch)
    shapes = [(512, 512)] * 6 + [(128, 1024)] * 4
    b, xs, d_in, _ = _plan(tctx, torch, shapes, (SHIFT,), inplace=True)
    res = b.autotune(None, reps=2, stream=s)
    torch.cuda.synchronize()
    for i, x in enumerate(xs):
        assert np.array_equal(d_in[i].cpu().numpy(), x)
    assert not res["from_cache"]
    b.execute(s)
    assert b.status(s) == 0
    for i in (0, 7):
        ref = oracle.fft2d(xs[i], SHIFT, 1)
        got = d_in[i].cpu().numpy()
        assert oracle.are_equal(ref, got, 64, oracle.fft_eps(max(shapes[i]), SHIFT) * 2) == 0
    b.close()
