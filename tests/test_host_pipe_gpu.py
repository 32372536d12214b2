"""gls::fft over images in host memory (glsfft_fft2d_host): chunks move
host -> device, through a batch plan, and back on three streams; the
results must be bit-identical to the device path, respect the caller's
stream order, survive shape changes and respect the context budget."""
from __future__ import annotations

import numpy as np
import pytest

import glscv_gb300 as g
from glscv_gb300 import workloads as wl
from tests.gpu_util import gpu_fft, stream_handle

pytestmark = pytest.mark.gpu

INV, SCALE, SHIFT = 1, 2, 64


def _host(torch, arr):
    return torch.from_numpy(np.ascontiguousarray(arr)).pin_memory()


@pytest.mark.parametrize("shape,count,chunk,flags", [
    ((256, 512), 10, 4, (0,)),          # two full chunks and a tail of two
    ((1024, 1024), 7, 0, (SHIFT,)),     # automatic chunk
    ((256, 256), 40, 0, (0, INV | SCALE)),  # automatic chunk (10 images), two transforms
    ((64, 2048), 9, 3, (INV | SCALE,)),
    ((2048, 2048), 3, 1, (0,)),         # images outside the persistent kernel
])
def test_host_pipeline_bit_identical_to_device_path(torch_cuda, shape, count, chunk, flags):
    torch = torch_cuda
    rows, cols = shape
    xs = np.stack([wl.complex_uniform(rows, cols, 1300 + i) for i in range(count)])
    h_in, h_out = _host(torch, xs), _host(torch, np.zeros_like(xs))
    with g.Context(0) as c:
        c.fft2d_host(h_in.data_ptr(), h_out.data_ptr(), count, rows, cols, flags, chunk,
                     stream_handle(torch))
        torch.cuda.synchronize()
        for i in range(count):
            ref = xs[i]
            for f in flags:  # the chain of transforms, one device call each
                ref = gpu_fft(c, torch, ref, f)
            assert np.array_equal(h_out[i].numpy().view(np.uint32), ref.view(np.uint32)), i
    assert np.array_equal(h_in.numpy(), xs)  # the input is left alone


def test_host_pipeline_round_trip_in_place_and_rebuild(torch_cuda, oracle):
    torch = torch_cuda
    s = stream_handle(torch)
    with g.Context(0) as c:
        for (rows, cols), count in (((1024, 1024), 6), ((128, 256), 40), ((1024, 1024), 6)):
            xs = np.stack([wl.complex_uniform(rows, cols, 1400 + i) for i in range(count)])
            h = _host(torch, xs)
            c.fft2d_host(h.data_ptr(), h.data_ptr(), count, rows, cols, (0, INV | SCALE), 0, s)
            torch.cuda.synchronize()
            for i in range(0, count, 5):
                assert oracle.rel_l2(h[i].numpy(), xs[i]) < 5e-7


def test_host_pipeline_follows_the_callers_stream(torch_cuda, oracle):
    """Work queued on the caller's stream before the call (here a device ->
    host copy that produces the input) completes before the upload."""
    torch = torch_cuda
    rows, cols, count = 512, 512, 4
    xs = np.stack([wl.complex_uniform(rows, cols, 1500 + i) for i in range(count)])
    d = torch.from_numpy(xs).cuda()
    h_in, h_out = _host(torch, np.zeros_like(xs)), _host(torch, np.zeros_like(xs))
    torch.cuda.synchronize()
    stream = torch.cuda.Stream()
    with g.Context(0) as c, torch.cuda.stream(stream):
        # a slow producer on the caller's stream, then the copy of the input
        for _ in range(20):
            d.mul_(1.0)
        h_in.copy_(d, non_blocking=True)
        c.fft2d_host(h_in.data_ptr(), h_out.data_ptr(), count, rows, cols, (0,), 1,
                     stream.cuda_stream)
        stream.synchronize()
        for i in range(count):
            ref = oracle.fft2d(xs[i], 0, 1)
            assert oracle.are_equal(ref, h_out[i].numpy(), 64, oracle.fft_eps(512, 0) * 2) == 0


def test_host_pipeline_respects_budget(torch_cuda):
    torch = torch_cuda
    xs = np.zeros((8, 1024, 1024), np.complex64)
    h = _host(torch, xs)
    with g.Context(0) as c:
        c.set_budget(16 << 20)  # less than three slots of two 8 MiB images
        with pytest.raises(g.GlsError) as e:
            c.fft2d_host(h.data_ptr(), h.data_ptr(), 8, 1024, 1024, (0,), 2, 0)
        assert e.value.status == 7
