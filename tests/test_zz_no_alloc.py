"""glsfft_phase_correlate_noalloc: phaseCorrelate without any device allocation.

This entry point is for callers that may not call cudaMalloc -- hosts whose
device memory belongs to their own pool or budget, and per-frame loops where
an allocation would synchronise the device.  Its scratch is a static device
array of the library, shared by every call.  The test calls it through the C
ABI twice in a row (a larger image, then a smaller one, so the second call
runs on a scratch array still holding the first call's data) and checks each
result against the context-based entry point: both run the same kernels with
the same twiddle table and scratch layout, so dx, dy, response, peak index and
peak value must be bit-identical (a stale-scratch or layout bug would move
them).  The integer peak must also equal the oracle's.  It also checks that
an image above the static limit is refused.  This file sorts last so a failing run has already run every other
test; it passes alone or after them.
"""
from __future__ import annotations

import numpy as np
import pytest

import glscv_gb300 as g
from glscv_gb300 import workloads as wl

pytestmark = pytest.mark.gpu

NOALLOC_LIMIT = 10
MAX_PIXELS = 512 * 512


def _noalloc(native, torch, a, b, w, box=5):
    rows, cols = a.shape
    res = torch.full((8,), float("nan"), dtype=torch.float64, device="cuda")
    st = native.glsfft_phase_correlate_noalloc(a.data_ptr(), b.data_ptr(),
                                              w.data_ptr() if w is not None else None,
                                              rows, cols, box, res.data_ptr(),
                                              torch.cuda.current_stream().cuda_stream)
    assert st == 0, native.glsfft_status_string(st)
    torch.cuda.synchronize()
    return res.cpu().numpy()


def _with_context(torch, a, b, w, box=5):
    rows, cols = a.shape
    res = torch.full((8,), float("nan"), dtype=torch.float64, device="cuda")
    with g.Context(0) as ctx:
        ctx.phase_correlate_async(a.data_ptr(), b.data_ptr(),
                                  w.data_ptr() if w is not None else None, rows, cols, box,
                                  res.data_ptr(), torch.cuda.current_stream().cuda_stream)
        torch.cuda.synchronize()
    return res.cpu().numpy()


def test_noalloc_matches_context_entry_point_two_calls(native, torch_cuda, oracle):
    torch = torch_cuda
    cases = [((512, 512), 41, (-40.4, 22.7), True), ((256, 256), 42, (17.0, -9.0), False)]
    for (rows, cols), seed, shift, use_window in cases:
        a, b = wl.random_pair(rows, cols, seed=seed, shift=shift)
        w = wl.hann_window(rows, cols) if use_window else None
        da, db = torch.from_numpy(a).cuda(), torch.from_numpy(b).cuda()
        dw = torch.from_numpy(w).cuda() if w is not None else None
        got = _noalloc(native, torch, da, db, dw)
        ref = _with_context(torch, da, db, dw)
        assert np.all(np.isfinite(got[:5]))
        # dx, dy, response, peak index, peak value: bit for bit
        assert np.array_equal(got[:5].view(np.uint64), ref[:5].view(np.uint64)), (got, ref)
        # the integer peak is the oracle's
        _, _, (px, py), _ = oracle.phase_correlate(a, b, w, box=5)
        assert int(got[3]) == py * cols + px
        assert abs(got[0] - shift[0]) < 0.5 and abs(got[1] - shift[1]) < 0.5


def test_noalloc_rejects_images_above_the_limit(native, torch_cuda):
    torch = torch_cuda
    d = torch.zeros((1024, 1024), dtype=torch.float32, device="cuda")
    res = torch.zeros(8, dtype=torch.float64, device="cuda")
    assert 1024 * 1024 > MAX_PIXELS
    st = native.glsfft_phase_correlate_noalloc(d.data_ptr(), d.data_ptr(), None, 1024, 1024, 5,
                                              res.data_ptr(), None)
    assert st == NOALLOC_LIMIT
    assert b"GLSFFT_NOALLOC_MAX_PIXELS" in native.glsfft_status_string(st)
