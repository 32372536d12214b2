"""The streamed column pass (pass schedule GLSFFT_SCHEDULE_STREAMED) on the GPU.

The streamed column pass of 2048- and 4096-point columns computes with the
plain kernels' arithmetic (same radix order, twiddles and rounding), so its
output must be bit-identical to schedule 0 -- for every gls::fft flag
combination (glsFft.h:43-47), batches of several images, in place
(glsPhaseCorrelate.cpp:199 calls fft(C, C)) and through the single-pass
entry point -- and arguments it cannot take (a buffer that is only 8-byte
aligned) must fall back to schedule 0.  No bounded wait may expire on the
way.  The built-in default schedules (row schedule 2 for 2048/4096-point
rows, the streamed pass for 4096-point columns) must equal schedule 0 bit
for bit as well.
"""
from __future__ import annotations

import numpy as np
import pytest

import glscv_gb300 as g
from glscv_gb300 import workloads as wl
from tests.gpu_util import stream_handle

pytestmark = pytest.mark.gpu

INV, SCALE, SHIFT = 1, 2, 64
STREAMED = 6
TIMEOUT = 8  # GLSFFT_ERROR_TIMEOUT


@pytest.fixture()
def tctx(native, torch_cuda):
    c = g.Context(0)
    yield c
    c.close()


def _run(ctx, torch, x, rows, cols, flags, count, sched, inplace=False):
    s = stream_handle(torch)
    ctx.set_fft_schedule(rows, cols, *sched)
    d = torch.from_numpy(x).cuda()
    out = d if inplace else torch.empty_like(d)
    if count == 1:
        ctx.fft2d(d.data_ptr(), out.data_ptr(), rows, cols, flags, s)
    else:
        ctx.fft2d_batched(d.data_ptr(), out.data_ptr(), count, rows, cols, flags, s)
    torch.cuda.synchronize()
    return out.cpu().numpy()


def _batch(rows, cols, count, seed):
    return np.stack([wl.complex_uniform(rows, cols, seed + i) for i in range(count)]) \
        if count > 1 else wl.complex_uniform(rows, cols, seed)


@pytest.mark.parametrize("rows,cols,count", [(4096, 4096, 1), (2048, 2048, 2), (2048, 1024, 3),
                                             (4096, 64, 2), (4096, 8, 1), (2048, 16, 2)])
@pytest.mark.parametrize("flags", [0, INV | SCALE, SHIFT, INV | SCALE | SHIFT])
def test_streamed_equals_schedule0(tctx, torch_cuda, rows, cols, count, flags):
    x = _batch(rows, cols, count, 1200 + rows + cols + flags)
    ref = _run(tctx, torch_cuda, x, rows, cols, flags, count, (0, 0))
    rs = 2 if g.schedule_available(cols, 2, False) else 0
    got = _run(tctx, torch_cuda, x, rows, cols, flags, count, (rs, STREAMED))
    assert np.array_equal(ref.view(np.uint32), got.view(np.uint32))
    got_ip = _run(tctx, torch_cuda, x, rows, cols, flags, count, (rs, STREAMED), inplace=True)
    assert np.array_equal(ref.view(np.uint32), got_ip.view(np.uint32))
    assert tctx.device_status() == 0


def test_streamed_matches_fp64(tctx, torch_cuda, oracle):
    x = wl.complex_uniform(4096, 4096, 1299)
    y = _run(tctx, torch_cuda, x, 4096, 4096, 0, 1, (0, STREAMED))
    ref64 = oracle.fft2d_f64(x)
    assert oracle.rel_l2(y, ref64) < 5e-7
    back = _run(tctx, torch_cuda, y, 4096, 4096, INV | SCALE, 1, (0, STREAMED))
    assert oracle.rel_l2(back, x) < 5e-7


def test_streamed_single_pass_entry_point(tctx, torch_cuda):
    torch = torch_cuda
    s = stream_handle(torch)
    rows, cols, count = 4096, 2048, 2
    x = _batch(rows, cols, count, 1310)
    d = torch.from_numpy(x).cuda()
    outs = []
    for sched in ((0, 0), (0, STREAMED)):
        tctx.set_fft_schedule(rows, cols, *sched)
        o = torch.empty_like(d)
        tctx.fft_cols(d.data_ptr(), o.data_ptr(), rows, cols, INV | SCALE | SHIFT, s, count)
        torch.cuda.synchronize()
        outs.append(o.cpu().numpy())
    assert np.array_equal(outs[0].view(np.uint32), outs[1].view(np.uint32))


def test_streamed_falls_back_on_8_byte_alignment(tctx, torch_cuda):
    torch = torch_cuda
    s = stream_handle(torch)
    n = 2048
    x = wl.complex_uniform(n, n, 1320)
    ref = _run(tctx, torch, x, n, n, 0, 1, (0, 0))
    # one extra complex value in front: the image starts 8 bytes into the buffer
    buf = torch.zeros(n * n + 1, dtype=torch.complex64, device="cuda")
    buf[1:] = torch.from_numpy(x.reshape(-1)).cuda()
    out = torch.zeros_like(buf)
    assert buf.data_ptr() % 16 == 0 and out.data_ptr() % 16 == 0
    tctx.set_fft_schedule(n, n, 0, STREAMED)
    tctx.fft2d(buf.data_ptr() + 8, out.data_ptr() + 8, n, n, 0, s)
    torch.cuda.synchronize()
    got = out[1:].cpu().numpy().reshape(ref.shape)
    assert np.array_equal(ref.view(np.uint32), got.view(np.uint32))
    assert tctx.device_status() == 0


def test_streamed_schedule_availability(native):
    for n in (2048, 4096):
        assert g.schedule_available(n, STREAMED, True)       # column pass
        assert not g.schedule_available(n, STREAMED, False)  # no row variant
    for n in (64, 1024):
        assert not g.schedule_available(n, STREAMED, True)


def test_builtin_default_schedules(tctx, torch_cuda):
    # a fresh context: 4096^2 runs row schedule 2 and the streamed column
    # pass, 2048-point rows schedule 2, other sizes schedule 0
    assert tctx.get_fft_schedule(4096, 4096) == (2, STREAMED)
    assert tctx.get_fft_schedule(2048, 2048) == (2, 0)
    assert tctx.get_fft_schedule(1024, 1024) == (0, 0)
    assert tctx.get_fft_schedule(4096, 1024) == (0, STREAMED)
    x = wl.complex_uniform(4096, 4096, 1330)
    s = stream_handle(torch_cuda)
    d = torch_cuda.from_numpy(x).cuda()
    y = torch_cuda.empty_like(d)
    tctx.fft2d(d.data_ptr(), y.data_ptr(), 4096, 4096, 0, s)       # the defaults
    torch_cuda.cuda.synchronize()
    ref = _run(tctx, torch_cuda, x, 4096, 4096, 0, 1, (0, 0))       # explicit schedule 0
    assert tctx.get_fft_schedule(4096, 4096) == (0, 0)
    assert np.array_equal(ref.view(np.uint32), y.cpu().numpy().view(np.uint32))
    tctx.set_fft_schedule(4096, 4096, 2, STREAMED)                  # back to the default
    assert tctx.get_fft_schedule(4096, 4096) == (2, STREAMED)


def test_streamed_stall_reports_timeout_and_context_recovers(tctx, torch_cuda):
    # fault injection on the host side: each block's first tile copy is never
    # issued, so its bounded wait (1 ms) runs out; the pass records
    # GLSFFT_ERROR_TIMEOUT and returns with no copy in flight, and the same
    # context then transforms correctly again
    n = 4096
    x = wl.complex_uniform(n, n, 1340)
    ref = _run(tctx, torch_cuda, x, n, n, 0, 1, (0, 0))
    assert tctx.device_status(clear=True) == 0
    tctx.inject_stall(1_000_000)
    _run(tctx, torch_cuda, x, n, n, 0, 1, (0, STREAMED))
    assert tctx.device_status(clear=True) == TIMEOUT
    assert tctx.device_status() == 0
    tctx.inject_stall(0)
    got = _run(tctx, torch_cuda, x, n, n, 0, 1, (0, STREAMED))
    assert tctx.device_status() == 0
    assert np.array_equal(ref.view(np.uint32), got.view(np.uint32))
