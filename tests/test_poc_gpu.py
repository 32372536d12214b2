"""gls::phaseCorrelate on the GPU through the C ABI, against the oracle.

* White-spectrum inputs (the reference test's uniform images,
  UnitTest_glsPhaseCorrelate.cpp:87): integer peak identical to the oracle's,
  sub-pixel shift within 1e-3 px of the oracle, response within 1e-4.
* Smooth-field inputs (Gaussian-blurred noise, the benchmark configuration):
  on about 46% of the bins of src1's spectrum any FP32 FFT's rounding error
  exceeds the bin's own magnitude, and the phase-only normalisation lifts
  those bins to unit magnitude with an implementation-specific phase.  The
  integer peak is still identical and must equal the true shift; the
  sub-pixel value is compared with the FP64 restatement of the whole
  pipeline over 8 seeds, against the distance the reference's own FP32
  arithmetic (the oracle) keeps from it.
* The ground truth (the synthetic shift) is met within the reference test's
  0.25 px (UnitTest_glsPhaseCorrelate.cpp:128-132).
"""
from __future__ import annotations

import numpy as np
import pytest

from glscv_gb300 import workloads as wl
from tests.gpu_util import gpu_phase_correlate

pytestmark = pytest.mark.gpu


def _peak(n_rows, n_cols, dx, dy):
    return (int(round(n_cols / 2 - dx)) % n_cols, int(round(n_rows / 2 - dy)) % n_rows)


@pytest.mark.parametrize("shape", [(32, 32), (64, 64), (256, 256), (1024, 1024), (64, 128),
                                   (512, 256), (2048, 2048)])
def test_white_spectrum_integer_shift(ctx, torch_cuda, oracle, shape):
    rows, cols = shape
    dx, dy = cols // 8 - 3, -(rows // 16) + 1
    a, b = wl.random_pair(rows, cols, seed=rows + cols, shift=(dx, dy))
    win = wl.hann_window(rows, cols)
    for w in (win, None):
        (ox, oy), oresp, opeak, osurf = oracle.phase_correlate(a, b, w, box=5, want_surface=True)
        (gx, gy), gresp, gsurf = gpu_phase_correlate(ctx, torch_cuda, a, b, w, box=5,
                                                     want_surface=True)
        (px, py), _ = oracle.max_loc(gsurf)
        assert (px, py) == opeak == _peak(rows, cols, dx, dy)
        assert abs(gx - ox) < 1e-3 and abs(gy - oy) < 1e-3
        assert abs(gresp - oresp) < 1e-4
        assert abs(gx - dx) < 0.25 and abs(gy - dy) < 0.25
        assert oracle.rel_l2(gsurf, osurf) < 1e-3


@pytest.mark.parametrize("box", [1, 3, 5, 7])
def test_subpixel_and_box(ctx, torch_cuda, oracle, box):
    n = 256
    a, b = wl.random_pair(n, n, seed=21, shift=(10.37, -5.62))
    win = wl.hann_window(n, n)
    (ox, oy), oresp, _, _ = oracle.phase_correlate(a, b, win, box=box)
    (gx, gy), gresp, _ = gpu_phase_correlate(ctx, torch_cuda, a, b, win, box=box)
    assert abs(gx - ox) < 1e-3 and abs(gy - oy) < 1e-3
    assert abs(gresp - oresp) < 1e-4


@pytest.mark.parametrize("n,max_shift", [(512, 30), (2048, 100)])
def test_smooth_field_config2b(ctx, torch_cuda, oracle, n, max_shift):
    """A = blurred noise (sigma 4 px) in [0,1], B = A rolled by an integer
    shift in [-max_shift, max_shift] + N(0, 0.01^2), Hann window.  The shift
    range is kept where the surface's highest value clears its neighbours by
    more than the FP32 noise floor: at 512 with a 45 px shift the top two
    values are 2% apart and the FP32 restatement itself picks the wrong
    neighbour."""
    a, b, (dx, dy) = wl.shifted_pair(n, n, seed_field=6, seed_shift=7, max_shift=max_shift)
    win = wl.hann_window(n, n)
    (ox, oy), oresp, opeak, _ = oracle.phase_correlate(a, b, win, box=5)
    (gx, gy), gresp, gsurf = gpu_phase_correlate(ctx, torch_cuda, a, b, win, box=5,
                                                 want_surface=True)
    (px, py), _ = oracle.max_loc(gsurf)
    assert (px, py) == opeak == _peak(n, n, dx, dy)
    # two FP32 implementations on a smooth field: see the 1024 test below
    assert abs(gx - ox) < 0.02 and abs(gy - oy) < 0.02
    assert abs(gx - dx) < 0.25 and abs(gy - dy) < 0.25


CONFIG_2B_SEEDS = [(6 + 100 * k, 7 + 100 * k) for k in range(8)]


def test_config2b_1024_against_fp64_pipeline(ctx, torch_cuda, oracle):
    """The benchmark phaseCorrelate (1024^2, shifts in [-100, 100], Hann
    window), 8 seeds, against the FP64 restatement of the whole pipeline
    (oracle.phase_correlate_f64: window product, complex128 DFTs, phase-only
    spectrum with the zero-bin guard, unscaled inverse, first maximum, FP64
    centroid).  Per seed: the integer peak equals the oracle's, the FP64
    pipeline's and the true shift; the sub-pixel shift is within 0.01 px of
    the oracle (measured: at most 0.0062 px over 12 seeds) and within 0.025 px
    of FP64 (the reference's FP32 arithmetic itself reaches 0.0173 px).  Over
    the seeds: the GPU's mean distance to FP64 is at most 1.25x the oracle's
    (measured 0.85x over these 8 seeds: the GPU is on average nearer to FP64
    than the reference's own FP32 arithmetic)."""
    torch = torch_cuda
    n = 1024
    win = wl.hann_window(n, n)
    d_gpu, d_orc = [], []
    for sf, ss in CONFIG_2B_SEEDS:
        a, b, (dx, dy) = wl.shifted_pair(n, n, seed_field=sf, seed_shift=ss, max_shift=100)
        (ox, oy), _, opeak, _ = oracle.phase_correlate(a, b, win, box=5)
        (fx, fy), _, fpeak, _ = oracle.phase_correlate_f64(a, b, win, box=5)
        (gx, gy), _, gsurf = gpu_phase_correlate(ctx, torch, a, b, win, box=5, want_surface=True)
        (px, py), _ = oracle.max_loc(gsurf)
        assert (px, py) == opeak == fpeak == _peak(n, n, dx, dy), (sf, ss)
        assert max(abs(gx - ox), abs(gy - oy)) <= 0.01, (sf, ss, (gx, gy), (ox, oy))
        dg = max(abs(gx - fx), abs(gy - fy))
        assert dg <= 0.025, (sf, ss, dg)
        d_gpu.append(dg)
        d_orc.append(max(abs(ox - fx), abs(oy - fy)))
    assert np.mean(d_gpu) <= 1.25 * np.mean(d_orc), (d_gpu, d_orc)


def test_identical_images_zero_shift(ctx, torch_cuda):
    n = 128
    a = np.random.default_rng(3).uniform(0, 1, (n, n)).astype(np.float32)
    (gx, gy), resp, _ = gpu_phase_correlate(ctx, torch_cuda, a, a, wl.hann_window(n, n))
    assert abs(gx) < 1e-6 and abs(gy) < 1e-6
    assert 0.5 < resp < 1.5


def test_constant_image_zero_bins_are_finite(ctx, torch_cuda):
    """All-zero cross spectrum except DC: the reference would produce NaN
    (0/0, glsBasicOperation.cpp:202-205); the GB300 path maps |t| = 0 to 0."""
    n = 64
    a = np.full((n, n), 0.5, np.float32)
    (gx, gy), resp, _ = gpu_phase_correlate(ctx, torch_cuda, a, a, None)
    assert np.isfinite(gx) and np.isfinite(gy) and np.isfinite(resp)


def test_async_matches_sync(ctx, torch_cuda, oracle):
    torch = torch_cuda
    n = 512
    a, b = wl.random_pair(n, n, seed=9, shift=(-33, 17))
    win = wl.hann_window(n, n)
    (gx, gy), gresp, _ = gpu_phase_correlate(ctx, torch, a, b, win)
    da, db, dw = (torch.from_numpy(v).cuda() for v in (a, b, win))
    res = torch.zeros(8, dtype=torch.float64, device="cuda")
    ctx.phase_correlate_async(da.data_ptr(), db.data_ptr(), dw.data_ptr(), n, n, 5,
                              res.data_ptr(), torch.cuda.current_stream().cuda_stream)
    r = res.cpu().numpy()
    assert r[0] == gx and r[1] == gy and r[2] == gresp
    assert int(r[3]) == (n // 2 - 17) * n + (n // 2 + 33)


def test_budget_error(native, torch_cuda):
    import glscv_gb300 as g
    torch = torch_cuda
    with g.Context(0) as c:
        c.set_budget(1024)
        d = torch.zeros((64, 64), dtype=torch.float32, device="cuda")
        with pytest.raises(g.GlsError) as e:
            c.phase_correlate(d.data_ptr(), d.data_ptr(), None, 64, 64)
        assert e.value.status == 7
        assert c.workspace_bytes() == 0


@pytest.mark.parametrize("shape,box,shift", [((256, 256), 5, (7.3, -4.6)),
                                             ((1024, 1024), 5, (-100.0, 37.0)),
                                             ((512, 256), 3, (11.5, 3.25)),
                                             ((64, 64), 7, (2.2, -1.7)),
                                             ((128, 128), 5, (64.0, 63.0)),      # box clamped
                                             ((2048, 2048), 5, (5.5, -5.5))])
def test_centroid_bit_exact_on_gpu_surface(ctx, torch_cuda, oracle, shape, box, shift):
    # on the GPU's own correlation surface, the first-max location and the
    # FP64 weighted centroid / response (separately rounded products and sums,
    # glsPhaseCorrelate.cpp:60-137, :205-231) equal the reference's
    # arithmetic bit for bit
    rows, cols = shape
    a, b = wl.random_pair(rows, cols, seed=rows + 3 * cols + box, shift=shift)
    win = wl.hann_window(rows, cols)
    (gx, gy), gresp, gsurf = gpu_phase_correlate(ctx, torch_cuda, a, b, win, box=box,
                                                 want_surface=True)
    (ox, oy), oresp, _ = oracle.centroid(gsurf, box)
    assert (gx, gy, gresp) == (ox, oy, oresp)


@pytest.mark.parametrize("n", [256, 1024])
def test_back_to_back_async_calls_match_synchronous(ctx, torch_cuda, n):
    # Eight asynchronous calls queued on one stream share the context's
    # workspace; each call's first pass overwrites the spectra its
    # predecessor's last pass reads, and the passes are chained by
    # programmatic dependent launch.  Every result must equal the same pair's
    # synchronous call, bit for bit.
    torch = torch_cuda
    from tests.gpu_util import stream_handle
    s = stream_handle(torch)
    w = torch.from_numpy(wl.hann_window(n, n)).cuda()
    pairs = []
    for i in range(8):
        a, b = wl.random_pair(n, n, seed=4000 + i, shift=(3.3 * i - 9.1, 11.7 - 2.2 * i))
        pairs.append((torch.from_numpy(np.ascontiguousarray(a, np.float32)).cuda(),
                      torch.from_numpy(np.ascontiguousarray(b, np.float32)).cuda()))
    res = torch.zeros((8, 8), dtype=torch.float64, device="cuda")
    for i, (da, db) in enumerate(pairs):
        ctx.phase_correlate_async(da.data_ptr(), db.data_ptr(), w.data_ptr(), n, n, 5,
                                  res[i].data_ptr(), s)
    torch.cuda.synchronize()
    got = res.cpu().numpy()
    for i, (da, db) in enumerate(pairs):
        (dx, dy), resp = ctx.phase_correlate(da.data_ptr(), db.data_ptr(), w.data_ptr(), n, n, 5, s)
        assert (got[i, 0], got[i, 1], got[i, 2]) == (dx, dy, resp)


def test_surface_discarded_by_a_later_workspace_user(ctx, torch_cuda, oracle):
    # the surface lives in the context workspace: a minMaxLoc that takes its
    # keys from the workspace overwrites it, and the copy is then refused
    import glscv_gb300 as g
    torch = torch_cuda
    a, b = wl.random_pair(64, 64, seed=4100, shift=(3.0, -2.0))
    (_, _), _, surf = gpu_phase_correlate(ctx, torch, a, b, None, box=5, want_surface=True)
    assert surf.shape == (64, 64)
    f = torch.rand(64, 64, device="cuda")
    ctx.min_max_loc(f.data_ptr(), 64, 64)
    d_surf = torch.empty((64, 64), dtype=torch.float32, device="cuda")
    with pytest.raises(g.GlsError):
        ctx.copy_surface(d_surf.data_ptr(), 64 * 64)


def test_async_call_captured_in_cuda_graph(ctx, torch_cuda):
    # the three chained launches captured into a CUDA graph (programmatic
    # dependencies become graph edges) and replayed give the synchronous result
    torch = torch_cuda
    n = 512
    a, b = wl.random_pair(n, n, seed=4200, shift=(12.4, -7.7))
    da = torch.from_numpy(np.ascontiguousarray(a, np.float32)).cuda()
    db = torch.from_numpy(np.ascontiguousarray(b, np.float32)).cuda()
    w = torch.from_numpy(wl.hann_window(n, n)).cuda()
    res = torch.zeros(8, dtype=torch.float64, device="cuda")
    side = torch.cuda.Stream()
    # first call outside the capture: workspace and kernel attributes are set up
    ctx.phase_correlate_async(da.data_ptr(), db.data_ptr(), w.data_ptr(), n, n, 5,
                              res.data_ptr(), side.cuda_stream)
    torch.cuda.synchronize()
    res.zero_()
    graph = torch.cuda.CUDAGraph()
    with torch.cuda.graph(graph, stream=side):
        ctx.phase_correlate_async(da.data_ptr(), db.data_ptr(), w.data_ptr(), n, n, 5,
                                  res.data_ptr(), side.cuda_stream)
    for _ in range(3):
        graph.replay()
    torch.cuda.synchronize()
    got = res.cpu().numpy()
    (dx, dy), resp = ctx.phase_correlate(da.data_ptr(), db.data_ptr(), w.data_ptr(), n, n, 5)
    assert (got[0], got[1], got[2]) == (dx, dy, resp)


@pytest.mark.parametrize("n", [256, 512, 1024])
def test_unaligned_frames_same_result(ctx, torch_cuda, n):
    """The windowed row pass stages 16-byte-aligned real frames of lines up
    to 512 points through shared memory with 16-byte loads and reads other
    frames element by element: frames 4 bytes past a 16-byte boundary give
    bit-identical results (and the promoted FFT of one the same spectrum)."""
    torch = torch_cuda
    a, b = wl.random_pair(n, n, seed=4300 + n, shift=(9.3, -4.6))
    w = torch.from_numpy(wl.hann_window(n, n)).cuda()
    out = []
    for off in (0, 1):
        da = torch.zeros(n * n + 4, dtype=torch.float32, device="cuda")
        db = torch.zeros(n * n + 4, dtype=torch.float32, device="cuda")
        da[off:off + n * n] = torch.from_numpy(np.ascontiguousarray(a, np.float32)).cuda().view(-1)
        db[off:off + n * n] = torch.from_numpy(np.ascontiguousarray(b, np.float32)).cuda().view(-1)
        pa, pb = da[off:].data_ptr(), db[off:].data_ptr()
        assert (pa % 16 == 0) == (off == 0)
        out.append(ctx.phase_correlate(pa, pb, w.data_ptr(), n, n, 5))
        spec = torch.empty((n, n), dtype=torch.complex64, device="cuda")
        ctx.fft2d(pa, spec.data_ptr(), n, n, 0, torch.cuda.current_stream().cuda_stream,
                  real_input=True)
        torch.cuda.synchronize()
        out.append(spec.cpu().numpy())
    assert out[0] == out[2]
    assert np.array_equal(out[1].view(np.uint32), out[3].view(np.uint32))


def test_sync_call_graph_cache_follows_buffers(ctx, torch_cuda):
    """The synchronous call replays a cached graph of its three launches
    while a call repeats the last one's buffers, shape and workspace.  A
    sequence that changes pairs, sizes and windows, and rewrites a buffer in
    place, must give the asynchronous path's result at every step."""
    torch = torch_cuda
    s = torch.cuda.current_stream().cuda_stream
    bufs = {}
    for name, n, seed in (("A", 256, 61), ("B", 256, 62), ("C", 512, 63)):
        a, b = wl.random_pair(n, n, seed=seed, shift=(5.4, -3.2))
        bufs[name] = (n, torch.from_numpy(np.ascontiguousarray(a, np.float32)).cuda(),
                      torch.from_numpy(np.ascontiguousarray(b, np.float32)).cuda(),
                      torch.from_numpy(wl.hann_window(n, n)).cuda())
    res = torch.zeros(8, dtype=torch.float64, device="cuda")

    def both(name, window=True, box=5):
        n, da, db, dw = bufs[name]
        w = dw.data_ptr() if window else None
        (dx, dy), resp = ctx.phase_correlate(da.data_ptr(), db.data_ptr(), w, n, n, box, s)
        ctx.phase_correlate_async(da.data_ptr(), db.data_ptr(), w, n, n, box, res.data_ptr(), s)
        torch.cuda.synchronize()
        got = res.cpu().numpy()
        assert (dx, dy, resp) == (got[0], got[1], got[2]), name

    for step in ("A", "A", "B", "A", "C", "C", "B"):
        both(step)
    both("A", window=False)
    both("A")
    both("A", box=3)
    both("A", box=7)
    both("A")
    # same pointers, new content: the replayed graph reads the buffers anew
    n, da, db, dw = bufs["A"]
    a2, b2 = wl.random_pair(n, n, seed=64, shift=(-7.1, 2.6))
    da.copy_(torch.from_numpy(np.ascontiguousarray(a2, np.float32)).cuda())
    db.copy_(torch.from_numpy(np.ascontiguousarray(b2, np.float32)).cuda())
    both("A")
    (dx, dy), _ = ctx.phase_correlate(da.data_ptr(), db.data_ptr(), dw.data_ptr(), n, n, 5, s)
    assert abs(abs(dx) - 7.1) < 0.5 and abs(abs(dy) - 2.6) < 0.5
