"""Helpers for gpu-marked tests: move numpy arrays through the C ABI."""
from __future__ import annotations

import numpy as np


def stream_handle(torch) -> int:
    return torch.cuda.current_stream().cuda_stream


def gpu_fft(ctx, torch, x: np.ndarray, flags: int = 0, inplace: bool = False) -> np.ndarray:
    """gls::fft through glsfft_fft2d_c2c (complex) or _r2c_promote (float32)."""
    rows, cols = x.shape
    real = x.dtype == np.float32
    d_in = torch.from_numpy(np.ascontiguousarray(x)).cuda()
    if inplace:
        assert not real
        d_out = d_in
    else:
        d_out = torch.empty((rows, cols), dtype=torch.complex64, device="cuda")
    ctx.fft2d(d_in.data_ptr(), d_out.data_ptr(), rows, cols, flags, stream_handle(torch),
              real_input=real)
    torch.cuda.synchronize()
    return d_out.cpu().numpy()


def gpu_phase_correlate(ctx, torch, a, b, window=None, box=5, want_surface=False):
    rows, cols = a.shape
    da = torch.from_numpy(np.ascontiguousarray(a, np.float32)).cuda()
    db = torch.from_numpy(np.ascontiguousarray(b, np.float32)).cuda()
    dw = torch.from_numpy(np.ascontiguousarray(window, np.float32)).cuda() if window is not None else None
    s = stream_handle(torch)
    (dx, dy), resp = ctx.phase_correlate(da.data_ptr(), db.data_ptr(),
                                         dw.data_ptr() if dw is not None else None,
                                         rows, cols, box, s)
    surf = None
    if want_surface:
        d_surf = torch.empty((rows, cols), dtype=torch.float32, device="cuda")
        ctx.copy_surface(d_surf.data_ptr(), rows * cols, s)
        torch.cuda.synchronize()
        surf = d_surf.cpu().numpy()
    return (dx, dy), resp, surf
