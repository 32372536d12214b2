"""Precision form: split-FP16 tensor-core four-step FFT (glsfft_fft2d_tc).

The bar is rel-L2 <= 1e-5 against an FP64 DFT, for uniform[-1,1] inputs and
for the 1e3 dynamic-range variant (magnitudes log-uniform in [1e-3, 1]),
with the FP32 CUDA-core path's error stated beside it; flags and batching
behave exactly like the FP32 path's.
"""
from __future__ import annotations

import numpy as np
import pytest

import glscv_gb300 as g
from glscv_gb300 import workloads as wl

pytestmark = pytest.mark.gpu

INV, SCALE, SHIFT = 1, 2, 64


def _run(ctx, torch, xs, flags, tc=True):
    d = torch.from_numpy(np.ascontiguousarray(np.stack(xs))).cuda()
    o = torch.empty_like(d)
    count, rows, cols = d.shape
    s = torch.cuda.current_stream().cuda_stream
    if tc:
        ctx.fft2d_tc(d.data_ptr(), o.data_ptr(), count, rows, cols, flags, s)
    else:
        ctx.fft2d_batched(d.data_ptr(), o.data_ptr(), count, rows, cols, flags, s)
    torch.cuda.synchronize()
    return o.cpu().numpy()


@pytest.mark.parametrize("shape", [(1024, 1024), (4096, 4096), (1024, 4096), (4096, 1024)])
@pytest.mark.parametrize("kind", ["uniform", "dynamic_range"])
def test_tc_error_vs_fp64(ctx, torch_cuda, oracle, shape, kind):
    rows, cols = shape
    gen = wl.complex_uniform if kind == "uniform" else wl.complex_dynamic_range
    x = gen(rows, cols, 4)
    y_tc = _run(ctx, torch_cuda, [x], 0)[0]
    y_32 = _run(ctx, torch_cuda, [x], 0, tc=False)[0]
    ref = oracle.fft2d_f64(x)
    e_tc, e_32 = oracle.rel_l2(y_tc, ref), oracle.rel_l2(y_32, ref)
    assert e_tc <= 1e-5, e_tc
    assert e_tc < 5 * e_32 + 1e-7, (e_tc, e_32)


@pytest.mark.parametrize("flags", [INV | SCALE, SHIFT, INV | SHIFT])
def test_tc_flags_and_batch_match_fp32_path(ctx, torch_cuda, oracle, flags):
    xs = [wl.complex_uniform(1024, 1024, 40 + i) for i in range(3)]
    y_tc = _run(ctx, torch_cuda, xs, flags)
    y_32 = _run(ctx, torch_cuda, xs, flags, tc=False)
    for i, x in enumerate(xs):
        assert oracle.rel_l2(y_tc[i], oracle.fft2d_f64(x, flags)) < 1e-6
        assert oracle.rel_l2(y_tc[i], y_32[i]) < 1e-6


def test_tc_rejects_other_sizes(ctx, torch_cuda):
    torch = torch_cuda
    d = torch.zeros((512, 512), dtype=torch.complex64, device="cuda")
    with pytest.raises(g.GlsError) as e:
        ctx.fft2d_tc(d.data_ptr(), d.data_ptr(), 1, 512, 512, 0)
    assert e.value.status == 3
