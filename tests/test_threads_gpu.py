"""Separate contexts used from separate host threads at the same time (the
C ABI's threading rule: a context per thread) give the same results as one
thread alone."""
from __future__ import annotations

import threading

import numpy as np
import pytest

import glscv_gb300 as g
from glscv_gb300 import workloads as wl

pytestmark = pytest.mark.gpu


def test_two_threads_two_contexts(torch_cuda):
    torch = torch_cuda
    n, reps = 512, 20
    xs = [wl.complex_uniform(n, n, 1600 + i) for i in range(2)]
    ref = []
    with g.Context(0) as c:
        for x in xs:
            d = torch.from_numpy(x).cuda()
            o = torch.empty_like(d)
            c.fft2d(d.data_ptr(), o.data_ptr(), n, n, 0, 0)
            torch.cuda.synchronize()
            ref.append(o.cpu().numpy())
    errors = []

    def worker(i):
        try:
            torch.cuda.set_device(0)
            stream = torch.cuda.Stream()
            with g.Context(0) as c, torch.cuda.stream(stream):
                d = torch.from_numpy(xs[i]).cuda()
                o = torch.empty_like(d)
                re = d.real.contiguous()  # kept alive for the calls below
                for _ in range(reps):
                    c.fft2d(d.data_ptr(), o.data_ptr(), n, n, 0, stream.cuda_stream)
                    (dx, dy), _ = c.phase_correlate(re.data_ptr(), re.data_ptr(), None, n, n, 5,
                                                    stream.cuda_stream)
                stream.synchronize()
                got = o.cpu().numpy()
                if not np.array_equal(got.view(np.uint32), ref[i].view(np.uint32)):
                    errors.append(f"thread {i}: fft differs")
                if abs(dx) > 1e-3 or abs(dy) > 1e-3:
                    errors.append(f"thread {i}: self-correlation shift ({dx}, {dy})")
        except Exception as e:  # surfaced below
            errors.append(f"thread {i}: {e!r}")

    ts = [threading.Thread(target=worker, args=(i,)) for i in range(2)]
    for t in ts:
        t.start()
    for t in ts:
        t.join(timeout=120)
    assert not errors, errors
