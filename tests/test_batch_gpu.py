"""Batch plans (persistent work-queue kernel + CUDA graph) on the GPU.

Each image of an uneven batch must come out bit-identical to the
single-image gls::fft path (the persistent kernel runs the same line FFTs),
including images routed outside the persistent launch.  Failure detection
is tested without a GPU fault: a host-injected impossible dependency makes
one bounded wait expire; the launch finishes and reports TIMEOUT.
"""
from __future__ import annotations

import numpy as np
import pytest

import glscv_gb300 as g
from glscv_gb300 import workloads as wl
from tests.gpu_util import gpu_fft

pytestmark = pytest.mark.gpu

INV, SCALE, SHIFT = 1, 2, 64


def _run_batch(ctx, torch, shapes, flags, seed0=700, inplace=False, variant=None):
    xs = [wl.complex_uniform(r, c, seed0 + i) for i, (r, c) in enumerate(shapes)]
    d_in = [torch.from_numpy(x).cuda() for x in xs]
    d_out = d_in if inplace else [torch.empty_like(d) for d in d_in]
    s = torch.cuda.current_stream().cuda_stream
    b = g.Batch(ctx, [d.data_ptr() for d in d_in], [d.data_ptr() for d in d_out], shapes, flags)
    if variant is not None:
        b.set_variant(variant)
    b.execute(s)
    assert b.status(s) == 0
    outs = [d.cpu().numpy() for d in d_out]
    return b, xs, d_in, d_out, outs


def _single(ctx, torch, x, flags):
    y = x
    for f in flags:
        y = gpu_fft(ctx, torch, y, f)
    return y


@pytest.mark.parametrize("variant", [0, 1, 2, 3])
@pytest.mark.parametrize("flags", [(0,), (0, INV | SCALE), (SHIFT,), (INV, SCALE | SHIFT)])
def test_uneven_batch_bit_identical_to_single_path(ctx, torch_cuda, flags, variant):
    torch = torch_cuda
    shapes = [(128, 128), (256, 256), (512, 512), (1024, 1024), (1024, 2048), (128, 128),
              (16, 4096), (64, 32), (2048, 64), (1, 256), (256, 1), (4096, 4096)]
    b, xs, _, _, outs = _run_batch(ctx, torch, shapes, flags, variant=variant)
    info = b.info()
    assert info["persistent_images"] == 8 and info["items"] > 0 and info["grid"] > 0
    for i, x in enumerate(xs):
        ref = _single(ctx, torch, x, flags)
        assert np.array_equal(outs[i].view(np.uint32), ref.view(np.uint32)), (i, shapes[i])
    b.close()


def test_config3_batch_vs_oracle_and_replay(ctx, torch_cuda, oracle):
    """64 images drawn like the 512-image configuration (seed 3), forward
    only: each vs the oracle at the reference test's bar; the graph replays
    to identical results."""
    torch = torch_cuda
    shapes = wl.batch_sizes(64, seed=3)
    b, xs, d_in, d_out, outs = _run_batch(ctx, torch, shapes, (0,))
    for i in range(0, 64, 9):
        r, c = shapes[i]
        ref = oracle.fft2d(xs[i], 0, 1)
        assert oracle.are_equal(ref, outs[i], 64, oracle.fft_eps(max(r, c), 0) * 2) == 0
        assert oracle.rel_l2(outs[i], oracle.fft2d_f64(xs[i])) < 1e-6
    s = torch.cuda.current_stream().cuda_stream
    b.execute(s)
    assert b.status(s) == 0
    for i in range(64):
        assert np.array_equal(d_out[i].cpu().numpy().view(np.uint32), outs[i].view(np.uint32))
    b.close()


@pytest.mark.parametrize("variant", [0, 1, 2, 3])
def test_inplace_round_trip_batch(ctx, torch_cuda, oracle, variant):
    torch = torch_cuda
    shapes = [(1024, 1024)] * 6 + [(256, 512)] * 5
    b, xs, _, _, outs = _run_batch(ctx, torch, shapes, (0, INV | SCALE), inplace=True,
                                   variant=variant)
    for i, x in enumerate(xs):
        assert oracle.rel_l2(outs[i], x) < 1e-6
    b.close()


@pytest.mark.parametrize("variant", [0, 1, 2, 3])
def test_injected_stall_times_out_and_context_survives(ctx, torch_cuda, oracle, variant):
    torch = torch_cuda
    shapes = [(256, 256)] * 4
    b, xs, _, d_out, _ = _run_batch(ctx, torch, shapes, (0, INV | SCALE), variant=variant)
    b.inject_stall(50_000_000)  # 50 ms deadline on a wait that can never be met
    s = torch.cuda.current_stream().cuda_stream
    b.execute(s)
    assert b.status(s) == 8  # GLSFFT_ERROR_TIMEOUT
    b.close()
    # the context and device still work
    x = wl.complex_uniform(64, 64, 1)
    y = gpu_fft(ctx, torch, x, 0)
    assert oracle.rel_l2(y, oracle.fft2d_f64(x)) < 1e-6


@pytest.mark.parametrize("inplace", [False, True])
@pytest.mark.parametrize("flags", [(0, INV | SCALE), (SHIFT,), (INV, SCALE | SHIFT)])
def test_column_tiled_workspace_same_results(ctx, torch_cuda, flags, inplace):
    """Images of 1024 rows with 16 <= cols <= 1024 get a column-tiled
    workspace (columns passes read one contiguous block from it; at 1024^2
    every intermediate stays there, later rows tiles loading as 128-byte-
    swizzled boxes); with a budget that leaves it out, the columns passes
    work in place in dst.  The results are bit-identical either way, and to
    the single-image path."""
    torch = torch_cuda
    shapes = [(1024, 1024), (512, 256), (16, 4096), (1024, 2048), (64, 32), (128, 128),
              (256, 16), (512, 2048), (1024, 512), (1024, 64), (1024, 16)]
    b, xs, _, _, with_ws = _run_batch(ctx, torch, shapes, flags, variant=3, inplace=inplace)
    tiled = [(r, c) for r, c in shapes if r == 1024 and c <= 1024]
    assert b.workspace() == {"tiled_images": len(tiled), "bytes": sum(8 * r * c for r, c in tiled)}
    b.close()
    ctx.set_budget(4 << 20)  # the plan's tables fit, the workspace does not
    try:
        b2, _, _, _, without = _run_batch(ctx, torch, shapes, flags, variant=3, inplace=inplace)
        assert b2.workspace() == {"tiled_images": 0, "bytes": 0}
        b2.close()
    finally:
        ctx.set_budget(0)
    for i, x in enumerate(xs):
        assert np.array_equal(with_ws[i].view(np.uint32), without[i].view(np.uint32)), shapes[i]
        ref = _single(ctx, torch, x, flags)
        assert np.array_equal(with_ws[i].view(np.uint32), ref.view(np.uint32)), shapes[i]


def test_variant_switch_on_a_workspace_plan(ctx, torch_cuda):
    """One plan with column-tiled workspaces executed under every variant in
    turn (the plain kernel ignores the workspace, the warp-specialised ones
    use it): the same bits each time."""
    torch = torch_cuda
    shapes = [(1024, 1024), (1024, 256), (256, 256)]
    b, xs, d_in, d_out, first = _run_batch(ctx, torch, shapes, (0, INV | SCALE), variant=3)
    assert b.workspace()["tiled_images"] == 2
    s = torch.cuda.current_stream().cuda_stream
    for v in (0, 1, 3, 2, 0, 3):
        for d in d_out:
            d.zero_()
        b.set_variant(v)
        b.execute(s)
        assert b.status(s) == 0
        for i, d in enumerate(d_out):
            assert np.array_equal(d.cpu().numpy().view(np.uint32), first[i].view(np.uint32)), (v, i)
    b.close()


def test_batch_argument_errors(ctx, torch_cuda):
    torch = torch_cuda
    d = torch.zeros((8, 8), dtype=torch.complex64, device="cuda")
    with pytest.raises(g.GlsError):
        g.Batch(ctx, [d.data_ptr()], [d.data_ptr()], [(8, 6)], (0,))
    with pytest.raises(g.GlsError):
        g.Batch(ctx, [d.data_ptr()], [d.data_ptr()], [(8, 8)], (0, 1, 2))
    with pytest.raises(g.GlsError):
        g.Batch(ctx, [d.data_ptr()], [d.data_ptr()], [(8, 8)], (4,))


def test_config3_full_512_round_trip_property(ctx, torch_cuda):
    """The full 512-image uneven batch (sizes drawn with seed 3) forward then
    INVERSE|SCALE through one plan: every image comes back within FP32
    round-trip error (a size-independent check at the full configuration)."""
    torch = torch_cuda
    shapes = wl.batch_sizes(512, seed=3)
    gen = torch.Generator(device="cuda")
    gen.manual_seed(3)
    xs = [torch.empty(sh, dtype=torch.complex64, device="cuda") for sh in shapes]
    for x in xs:
        x.view(torch.float32).uniform_(-1, 1, generator=gen)
    outs = [torch.empty_like(x) for x in xs]
    s = torch.cuda.current_stream().cuda_stream
    b = g.Batch(ctx, [x.data_ptr() for x in xs], [o.data_ptr() for o in outs], shapes,
                (0, INV | SCALE))
    assert b.info()["persistent_images"] == 512
    b.execute(s)
    assert b.status(s) == 0
    worst = max(float(torch.linalg.vector_norm(o - x) / torch.linalg.vector_norm(x))
                for x, o in zip(xs, outs))
    assert worst < 5e-7, worst
    b.close()


def test_two_plans_concurrently_on_two_streams(ctx, torch_cuda):
    """Two persistent launches sized for the whole GPU, queued on two streams at
    once: blocks of the second start only as the first's retire, and dynamic
    claiming keeps both correct (no block ever holds an item another waits on
    without running)."""
    torch = torch_cuda
    shapes_a = [(512, 512)] * 24
    shapes_b = wl.batch_sizes(48, seed=5)
    plans, ins, outs, refs = [], [], [], []
    for shapes, seed in ((shapes_a, 1700), (shapes_b, 1800)):
        b, xs, d_in, d_out, _ = _run_batch(ctx, torch, shapes, (0, INV | SCALE), seed0=seed)
        plans.append(b)
        ins.append(d_in)  # the plans keep raw pointers: keep the buffers alive
        outs.append(d_out)
        refs.append([d.cpu().numpy().copy() for d in d_out])
        for d in d_out:
            d.zero_()
    torch.cuda.synchronize()
    s1, s2 = torch.cuda.Stream(), torch.cuda.Stream()
    for _ in range(3):
        plans[0].execute(s1.cuda_stream)
        plans[1].execute(s2.cuda_stream)
    torch.cuda.synchronize()
    assert plans[0].status(s1.cuda_stream) == 0 and plans[1].status(s2.cuda_stream) == 0
    for k in range(2):
        for i, d in enumerate(outs[k]):
            assert np.array_equal(d.cpu().numpy().view(np.uint32), refs[k][i].view(np.uint32)), (k, i)
    for b in plans:
        b.close()
