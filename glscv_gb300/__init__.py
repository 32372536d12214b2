"""glscv_gb300 -- GB300-native FFT / phaseCorrelate path of glsCV.

The product is the native library ``glscv_gb300/lib/libglscv_gb300.so``
(hand-written sm_103a CUDA kernels behind the C ABI of ``include/glsfft.h``
and the C++ ``gls::`` API of ``include/gls/glsCV.h``).  This module is a thin
ctypes binding used by the tests and the benchmark; it never falls back to
any other implementation: if the library is missing it raises.

Device buffers are passed as integer addresses (e.g. ``tensor.data_ptr()``);
streams as integer ``cudaStream_t`` handles (0 = legacy default stream).
"""
from __future__ import annotations

import ctypes
from pathlib import Path

__all__ = [
    "lib", "GlsError", "Context", "DFT_INVERSE", "DFT_SCALE", "GLS_FFT_SHIFT",
    "GLS_FFT_INVERSE", "GLS_FFT_SCALE", "LIB_PATH", "HEADER_PATHS", "schedule_available",
]

PKG = Path(__file__).resolve().parent
LIB_PATH = PKG / "lib" / "libglscv_gb300.so"
HEADER_PATHS = sorted((PKG.parent / "include").rglob("*.h"))

# flag values of the reference (glsCV/glsFft.h:43-47)
DFT_INVERSE = GLS_FFT_INVERSE = 1
DFT_SCALE = GLS_FFT_SCALE = 2
GLS_FFT_SHIFT = 64
# OR into the algo of phase_correlate_reference: |F1 conj F2| = 0 gives 0, not NaN
REFERENCE_ZERO_GUARD = 16

_vp = ctypes.c_void_p
_ip = ctypes.c_int
_sz = ctypes.c_size_t
_dp = ctypes.POINTER(ctypes.c_double)

_SIGNATURES = {
    "glsfft_status_string": (ctypes.c_char_p, [_ip]),
    "glsfft_version": (_ip, []),
    "glsfft_context_create": (_ip, [ctypes.POINTER(_vp), _ip]),
    "glsfft_context_destroy": (_ip, [_vp]),
    "glsfft_context_set_budget": (_ip, [_vp, _sz]),
    "glsfft_context_workspace": (_ip, [_vp, ctypes.POINTER(_sz)]),
    "glsfft_device_status": (_ip, [_vp, _ip]),
    "glsfft_context_inject_stall": (_ip, [_vp, ctypes.c_longlong]),
    "glsfft_fft2d_reference": (_ip, [_vp, _vp, _vp, _ip, _ip, _ip, _ip, _ip, _vp]),
    "glsfft_phase_correlate_reference": (_ip, [_vp, _vp, _vp, _vp, _ip, _ip, _ip, _ip,
                                               ctypes.POINTER(ctypes.c_double),
                                               ctypes.POINTER(ctypes.c_double),
                                               ctypes.POINTER(ctypes.c_double), _vp]),
    "glsfft_fft2d_c2c": (_ip, [_vp, _vp, _vp, _ip, _ip, _ip, _vp]),
    "glsfft_fft2d_r2c_promote": (_ip, [_vp, _vp, _vp, _ip, _ip, _ip, _vp]),
    "glsfft_fft_rows": (_ip, [_vp, _vp, _vp, _ip, _ip, _ip, _ip, _vp]),
    "glsfft_fft_cols": (_ip, [_vp, _vp, _vp, _ip, _ip, _ip, _ip, _vp]),
    "glsfft_fft2d_batched": (_ip, [_vp, _vp, _vp, _ip, _ip, _ip, _ip, _vp]),
    "glsfft_fft2d_tc": (_ip, [_vp, _vp, _vp, _ip, _ip, _ip, _ip, _vp]),
    "glsfft_fft2d_host": (_ip, [_vp, _vp, _vp, _ip, _ip, _ip, _ip, ctypes.POINTER(_ip), _ip, _vp]),
    "glsfft_mul_spectrums": (_ip, [_vp, _vp, _vp, _vp, _ip, _ip, _ip, _vp]),
    "glsfft_mul_spectrums_phase_only": (_ip, [_vp, _vp, _vp, _vp, _ip, _ip, _vp]),
    "glsfft_mag_spectrums": (_ip, [_vp, _vp, _vp, _ip, _ip, _vp]),
    "glsfft_log_mag_spectrums": (_ip, [_vp, _vp, _vp, _ip, _ip, ctypes.c_float, _vp]),
    "glsfft_min_max_loc": (_ip, [_vp, _vp, _ip, _ip, _dp, _dp, ctypes.POINTER(_ip),
                                 ctypes.POINTER(_ip), _vp]),
    "glsfft_min_max_loc_async": (_ip, [_vp, _vp, _ip, _ip, _vp, _vp]),
    "glsfft_normalize_minmax": (_ip, [_vp, _vp, _vp, _ip, _ip, ctypes.c_double, ctypes.c_double,
                                      _vp]),
    "glsfft_fft_display": (_ip, [_vp, _vp, _vp, _vp, _ip, _ip, ctypes.c_float, _vp]),
    "glsfft_phase_correlate": (_ip, [_vp, _vp, _vp, _vp, _ip, _ip, _ip, _dp, _dp, _dp, _vp]),
    "glsfft_phase_correlate_async": (_ip, [_vp, _vp, _vp, _vp, _ip, _ip, _ip, _vp, _vp]),
    "glsfft_phase_correlate_surface": (_ip, [_vp, _vp, _sz, _vp]),
    "glsfft_phase_correlate_noalloc": (_ip, [_vp, _vp, _vp, _ip, _ip, _ip, _vp, _vp]),
    "glsfft_batch_create": (_ip, [_vp, _ip, ctypes.POINTER(_vp), ctypes.POINTER(_vp),
                                  ctypes.POINTER(_ip), ctypes.POINTER(_ip), _ip,
                                  ctypes.POINTER(_ip), ctypes.POINTER(_vp)]),
    "glsfft_batch_execute": (_ip, [_vp, _vp]),
    "glsfft_batch_set_variant": (_ip, [_vp, _ip]),
    "glsfft_batch_set_schedule": (_ip, [_vp, _ip, _ip, _ip]),
    "glsfft_batch_status": (_ip, [_vp, _vp]),
    "glsfft_batch_info": (_ip, [_vp, ctypes.POINTER(_ip), ctypes.POINTER(_ip),
                                ctypes.POINTER(_ip)]),
    "glsfft_batch_workspace": (_ip, [_vp, ctypes.POINTER(_ip), ctypes.POINTER(_sz)]),
    "glsfft_batch_inject_stall": (_ip, [_vp, ctypes.c_longlong]),
    "glsfft_batch_get_schedule": (_ip, [_vp, ctypes.POINTER(_ip)]),
    "glsfft_batch_tuning": (_ip, [_vp, _ip, ctypes.POINTER(_ip), _dp, ctypes.POINTER(_ip)]),
    "glsfft_batch_set_stats": (_ip, [_vp, _ip]),
    "glsfft_batch_get_stats": (_ip, [_vp, _vp, _dp]),
    "glsfft_batch_autotune": (_ip, [_vp, ctypes.c_char_p, _ip, _vp, ctypes.POINTER(_ip), _dp]),
    "glsfft_schedule_available": (_ip, [_ip, _ip, _ip]),
    "glsfft_set_fft_schedule": (_ip, [_vp, _ip, _ip, _ip, _ip]),
    "glsfft_get_fft_schedule": (_ip, [_vp, _ip, _ip, ctypes.POINTER(_ip), ctypes.POINTER(_ip)]),
    "glsfft_autotune_fft2d": (_ip, [_vp, _ip, _ip, _ip, ctypes.c_char_p, _vp,
                                    ctypes.POINTER(_ip), _dp]),
    "glsfft_batch_destroy": (_ip, [_vp]),
    "glsfft_server_create": (_ip, [_vp, _ip, _sz, ctypes.POINTER(_vp)]),
    "glsfft_server_add_reference": (_ip, [_vp, _vp, _vp, _ip, _ip, ctypes.POINTER(_ip)]),
    "glsfft_server_submit": (_ip, [_vp, _ip, _vp, _ip, ctypes.POINTER(ctypes.c_longlong)]),
    "glsfft_server_wait": (_ip, [_vp, ctypes.c_longlong, _dp, _dp, ctypes.c_double]),
    "glsfft_server_replay": (_ip, [_vp, _ip, _dp, ctypes.POINTER(_ip), ctypes.POINTER(_vp), _ip,
                                   _dp, _dp]),
    "glsfft_server_replay_traced": (_ip, [_vp, _ip, _dp, ctypes.POINTER(_ip), ctypes.POINTER(_vp),
                                          _ip, _dp, _dp, _dp]),
    "glsfft_server_set_frame_read": (_ip, [_vp, _ip]),
    "glsfft_server_stats": (_ip, [_vp, ctypes.POINTER(ctypes.c_longlong)]),
    "glsfft_server_destroy": (_ip, [_vp]),
}

_lib = None


class GlsError(RuntimeError):
    """A non-zero status from the C ABI (the reference throws cv::Exception)."""

    def __init__(self, status: int, where: str = ""):
        self.status = status
        msg = lib().glsfft_status_string(status).decode()
        super().__init__(f"{where}: {msg} (status {status})" if where else msg)


def lib() -> ctypes.CDLL:
    """Load the native library (raises if it has not been built)."""
    global _lib
    if _lib is None:
        if not LIB_PATH.exists():
            raise RuntimeError(
                f"{LIB_PATH} is missing: build it with `python -m glscv_gb300.build` "
                "(there is no fallback implementation)")
        l = ctypes.CDLL(str(LIB_PATH))
        for name, (res, args) in _SIGNATURES.items():
            fn = getattr(l, name)
            fn.restype = res
            fn.argtypes = args
        _lib = l
    return _lib


def check(status: int, where: str = "") -> None:
    if status != 0:
        raise GlsError(status, where)


class Context:
    """Owns a glsfft_context (twiddle tables + workspace) on one device."""

    def __init__(self, device: int = 0):
        self.handle = _vp()
        check(lib().glsfft_context_create(ctypes.byref(self.handle), int(device)),
              "glsfft_context_create")
        self.device = device

    def close(self) -> None:
        if self.handle:
            lib().glsfft_context_destroy(self.handle)
            self.handle = _vp()

    def __enter__(self):
        return self

    def __exit__(self, *exc):
        self.close()

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    # -- gls::fft --------------------------------------------------------
    def fft2d(self, src: int, dst: int, rows: int, cols: int, flags: int = 0,
              stream: int = 0, real_input: bool = False) -> None:
        fn = lib().glsfft_fft2d_r2c_promote if real_input else lib().glsfft_fft2d_c2c
        check(fn(self.handle, src, dst, rows, cols, flags, stream), "fft2d")

    def fft2d_batched(self, src: int, dst: int, count: int, rows: int, cols: int,
                      flags: int = 0, stream: int = 0) -> None:
        check(lib().glsfft_fft2d_batched(self.handle, src, dst, count, rows, cols, flags, stream),
              "fft2d_batched")

    def fft2d_reference(self, src: int, dst: int, rows: int, cols: int, flags: int = 0,
                        algo: int = 0, stream: int = 0, count: int = 1) -> None:
        """Reference-arithmetic gls::fft (bit-identical to the reference's CPU
        Stockham: algo 0 radix-2 type1, 1 radix-4 lines)."""
        check(lib().glsfft_fft2d_reference(self.handle, src, dst, count, rows, cols, flags, algo,
                                           stream), "fft2d_reference")

    def phase_correlate_reference(self, src1: int, src2: int, window: int | None, rows: int,
                                  cols: int, box: int = 5, algo: int = 0, stream: int = 0):
        dx, dy, resp = ctypes.c_double(), ctypes.c_double(), ctypes.c_double()
        check(lib().glsfft_phase_correlate_reference(self.handle, src1, src2, window or None,
                                                     rows, cols, box, algo, ctypes.byref(dx),
                                                     ctypes.byref(dy), ctypes.byref(resp),
                                                     stream), "phase_correlate_reference")
        return (dx.value, dy.value), resp.value

    def fft2d_tc(self, src: int, dst: int, count: int, rows: int, cols: int, flags: int = 0,
                 stream: int = 0) -> None:
        """Precision form: split-FP16 tensor-core four-step FFT (1024/4096 lines)."""
        check(lib().glsfft_fft2d_tc(self.handle, src, dst, count, rows, cols, flags, stream),
              "fft2d_tc")

    def fft_rows(self, src: int, dst: int, rows: int, cols: int, flags: int = 0,
                 stream: int = 0, count: int = 1) -> None:
        check(lib().glsfft_fft_rows(self.handle, src, dst, count, rows, cols, flags, stream),
              "fft_rows")

    def fft_cols(self, src: int, dst: int, rows: int, cols: int, flags: int = 0,
                 stream: int = 0, count: int = 1) -> None:
        check(lib().glsfft_fft_cols(self.handle, src, dst, count, rows, cols, flags, stream),
              "fft_cols")

    # -- gls::phaseCorrelate -------------------------------------------------
    def phase_correlate(self, src1: int, src2: int, window: int | None, rows: int, cols: int,
                        box: int = 5, stream: int = 0):
        dx, dy, resp = ctypes.c_double(), ctypes.c_double(), ctypes.c_double()
        check(lib().glsfft_phase_correlate(self.handle, src1, src2, window or None, rows, cols,
                                           box, ctypes.byref(dx), ctypes.byref(dy),
                                           ctypes.byref(resp), stream), "phase_correlate")
        return (dx.value, dy.value), resp.value

    def phase_correlate_async(self, src1: int, src2: int, window: int | None, rows: int,
                              cols: int, box: int, d_result: int, stream: int = 0) -> None:
        check(lib().glsfft_phase_correlate_async(self.handle, src1, src2, window or None, rows,
                                                 cols, box, d_result, stream),
              "phase_correlate_async")

    def copy_surface(self, dst: int, count: int, stream: int = 0) -> None:
        check(lib().glsfft_phase_correlate_surface(self.handle, dst, count, stream), "surface")

    def workspace_bytes(self) -> int:
        b = _sz()
        check(lib().glsfft_context_workspace(self.handle, ctypes.byref(b)), "workspace")
        return b.value

    def device_status(self, clear: bool = False) -> int:
        """Sticky status of the context's device-side bounded waits (0 = none
        expired); synchronises with the device."""
        return int(lib().glsfft_device_status(self.handle, int(clear)))

    def inject_stall(self, wait_limit_ns: int) -> None:
        """Fault injection for tests: streamed passes leave their first tile
        copies unissued and time out after wait_limit_ns (0: off)."""
        check(lib().glsfft_context_inject_stall(self.handle, int(wait_limit_ns)), "inject_stall")

    def set_budget(self, nbytes: int) -> None:
        check(lib().glsfft_context_set_budget(self.handle, nbytes), "set_budget")

    def fft2d_host(self, host_src: int, host_dst: int, count: int, rows: int, cols: int,
                   flags=(0,), chunk: int = 0, stream: int = 0) -> None:
        """glsfft_fft2d_host: host images through 1-2 transforms, copies
        pipelined against the transforms (asynchronous on `stream`)."""
        fl = (_ip * len(flags))(*[int(f) for f in flags])
        check(lib().glsfft_fft2d_host(self.handle, host_src, host_dst, count, rows, cols,
                                      len(flags), fl, chunk, stream), "fft2d_host")

    # ---- spectrum operations, minMaxLoc, normalize, the FFT display pipeline
    def mul_spectrums(self, src0: int, src1: int, dst: int, rows: int, cols: int,
                      conj: bool = False, stream: int = 0) -> None:
        check(lib().glsfft_mul_spectrums(self.handle, src0, src1, dst, rows, cols, int(conj),
                                         stream), "mul_spectrums")

    def mul_spectrums_phase_only(self, src0: int, src1: int, dst: int, rows: int, cols: int,
                                 stream: int = 0) -> None:
        check(lib().glsfft_mul_spectrums_phase_only(self.handle, src0, src1, dst, rows, cols,
                                                    stream), "mul_spectrums_phase_only")

    def mag_spectrums(self, src: int, dst: int, rows: int, cols: int, stream: int = 0) -> None:
        check(lib().glsfft_mag_spectrums(self.handle, src, dst, rows, cols, stream),
              "mag_spectrums")

    def log_mag_spectrums(self, src: int, dst: int, rows: int, cols: int, offset: float,
                          stream: int = 0) -> None:
        check(lib().glsfft_log_mag_spectrums(self.handle, src, dst, rows, cols, offset, stream),
              "log_mag_spectrums")

    def min_max_loc(self, src: int, rows: int, cols: int, stream: int = 0):
        """((min, max), (min_x, min_y), (max_x, max_y)), synchronous."""
        mn, mx = ctypes.c_double(), ctypes.c_double()
        lmin, lmax = (_ip * 2)(), (_ip * 2)()
        check(lib().glsfft_min_max_loc(self.handle, src, rows, cols, ctypes.byref(mn),
                                       ctypes.byref(mx), lmin, lmax, stream), "min_max_loc")
        return (mn.value, mx.value), (lmin[0], lmin[1]), (lmax[0], lmax[1])

    def normalize_minmax(self, src: int, dst: int, rows: int, cols: int, alpha: float = 0.0,
                         beta: float = 1.0, stream: int = 0) -> None:
        check(lib().glsfft_normalize_minmax(self.handle, src, dst, rows, cols, alpha, beta,
                                            stream), "normalize_minmax")

    def fft_display(self, frame: int, window: int | None, dst: int, rows: int, cols: int,
                    offset: float = 1.0, stream: int = 0) -> None:
        check(lib().glsfft_fft_display(self.handle, frame, window, dst, rows, cols, offset,
                                       stream), "fft_display")

    def set_fft_schedule(self, rows: int, cols: int, row_schedule: int, col_schedule: int) -> None:
        check(lib().glsfft_set_fft_schedule(self.handle, rows, cols, row_schedule, col_schedule),
              "set_fft_schedule")

    def get_fft_schedule(self, rows: int, cols: int) -> tuple[int, int]:
        r, c = _ip(), _ip()
        check(lib().glsfft_get_fft_schedule(self.handle, rows, cols, ctypes.byref(r),
                                            ctypes.byref(c)), "get_fft_schedule")
        return r.value, c.value

    def autotune_fft2d(self, rows: int, cols: int, count: int = 1, cache_path: str | None = None,
                       stream: int = 0) -> dict:
        res = (_ip * 3)()
        ms = (ctypes.c_double * 2)()
        path = cache_path.encode() if cache_path else None
        check(lib().glsfft_autotune_fft2d(self.handle, rows, cols, count, path, stream, res, ms),
              "autotune_fft2d")
        return {"row_schedule": res[0], "col_schedule": res[1], "from_cache": bool(res[2]),
                "ms": ms[0], "ms_default": ms[1]}


def schedule_available(length: int, schedule: int, along_cols: bool) -> bool:
    return bool(lib().glsfft_schedule_available(length, schedule, int(along_cols)))


class Batch:
    """A batch plan (glsfft_batch): uneven-size images through 1-2 transforms,
    one persistent launch, captured into a CUDA graph."""

    def __init__(self, ctx: Context, srcs, dsts, shapes, flags=(0,)):
        n = len(srcs)
        self.handle = _vp()
        arr_v = _vp * n
        arr_i = _ip * n
        rows = arr_i(*[int(r) for r, _ in shapes])
        cols = arr_i(*[int(c) for _, c in shapes])
        fl = (_ip * len(flags))(*[int(f) for f in flags])
        check(lib().glsfft_batch_create(ctx.handle, n, arr_v(*srcs), arr_v(*dsts), rows, cols,
                                        len(flags), fl, ctypes.byref(self.handle)),
              "glsfft_batch_create")

    def execute(self, stream: int = 0) -> None:
        check(lib().glsfft_batch_execute(self.handle, stream), "batch_execute")

    def set_variant(self, variant: int) -> None:
        check(lib().glsfft_batch_set_variant(self.handle, int(variant)), "batch_set_variant")

    def set_schedule(self, claim_chunk: int = 1, claim_ahead: int = 0,
                     lag_items: int = 0) -> None:
        check(lib().glsfft_batch_set_schedule(self.handle, int(claim_chunk), int(claim_ahead),
                                              int(lag_items)), "batch_set_schedule")

    def status(self, stream: int = 0) -> int:
        return int(lib().glsfft_batch_status(self.handle, stream))

    def info(self):
        a, b, c = _ip(), _ip(), _ip()
        check(lib().glsfft_batch_info(self.handle, ctypes.byref(a), ctypes.byref(b),
                                      ctypes.byref(c)), "batch_info")
        return {"persistent_images": a.value, "items": b.value, "grid": c.value}

    def workspace(self):
        """glsfft_batch_workspace: images with a column-tiled workspace and
        the bytes the plan holds for them."""
        n, b = _ip(), _sz()
        check(lib().glsfft_batch_workspace(self.handle, ctypes.byref(n), ctypes.byref(b)),
              "batch_workspace")
        return {"tiled_images": n.value, "bytes": b.value}

    def inject_stall(self, wait_limit_ns: int) -> None:
        check(lib().glsfft_batch_inject_stall(self.handle, int(wait_limit_ns)), "inject_stall")

    def schedule(self) -> dict:
        out = (_ip * 4)()
        check(lib().glsfft_batch_get_schedule(self.handle, out), "batch_get_schedule")
        return {"variant": out[0], "claim_chunk": out[1], "claim_ahead": out[2],
                "lag_items": out[3]}

    def tuning(self) -> list[dict]:
        """Candidates of the last timed autotune: schedule and median ms."""
        n = _ip()
        check(lib().glsfft_batch_tuning(self.handle, 0, None, None, ctypes.byref(n)), "tuning")
        sch = (_ip * (4 * n.value))()
        ms = (ctypes.c_double * n.value)()
        check(lib().glsfft_batch_tuning(self.handle, n.value, sch, ms, ctypes.byref(n)), "tuning")
        return [{"variant": sch[4 * i], "claim_chunk": sch[4 * i + 1],
                 "claim_ahead": sch[4 * i + 2], "lag_grids": sch[4 * i + 3], "ms": ms[i]}
                for i in range(n.value)]

    def set_stats(self, on: bool) -> None:
        check(lib().glsfft_batch_set_stats(self.handle, int(on)), "batch_set_stats")

    def stats(self, stream: int = 0) -> dict:
        out = (ctypes.c_double * 8)()
        check(lib().glsfft_batch_get_stats(self.handle, stream, out), "batch_get_stats")
        keys = ["dep_wait_ns", "refill_wait_ns", "publish_wait_ns", "producer_ns",
                "full_wait_ns", "compute_ns", "items", "blocks"]
        return dict(zip(keys, list(out)))

    def autotune(self, cache_path: str | None = None, reps: int = 5, stream: int = 0) -> dict:
        res = (_ip * 6)()
        ms = (ctypes.c_double * 2)()
        path = cache_path.encode() if cache_path else None
        check(lib().glsfft_batch_autotune(self.handle, path, reps, stream, res, ms),
              "batch_autotune")
        return {"variant": res[0], "claim_chunk": res[1], "claim_ahead": res[2],
                "lag_items": res[3], "from_cache": bool(res[4]), "candidates": res[5],
                "ms": ms[0], "ms_default": ms[1]}

    def close(self) -> None:
        if self.handle:
            lib().glsfft_batch_destroy(self.handle)
            self.handle = _vp()

    def __enter__(self):
        return self

    def __exit__(self, *exc):
        self.close()

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass


class Server:
    """phaseCorrelate serving loop (glsfft_server): resident reference
    spectra, HBM-budget admission, continuous batching over `slots` streams."""

    STATS = ("admitted", "completed", "failed", "peak_in_flight", "peak_queue",
             "budget_bytes", "peak_budget_bytes", "references")

    def __init__(self, ctx: Context, slots: int = 8, hbm_budget: int = 4 << 30):
        self.handle = _vp()
        check(lib().glsfft_server_create(ctx.handle, int(slots), int(hbm_budget),
                                         ctypes.byref(self.handle)), "glsfft_server_create")

    def add_reference(self, frame: int, window: int | None, rows: int, cols: int) -> int:
        rid = _ip()
        check(lib().glsfft_server_add_reference(self.handle, frame, window or None, rows, cols,
                                                ctypes.byref(rid)), "server_add_reference")
        return rid.value

    def submit(self, ref_id: int, host_frame: int, box: int = 5) -> int:
        t = ctypes.c_longlong()
        check(lib().glsfft_server_submit(self.handle, int(ref_id), host_frame, int(box),
                                         ctypes.byref(t)), "server_submit")
        return t.value

    def wait(self, ticket: int, timeout_s: float = 30.0):
        res = (ctypes.c_double * 5)()
        lat = ctypes.c_double()
        check(lib().glsfft_server_wait(self.handle, ctypes.c_longlong(ticket),
                                       ctypes.cast(res, _dp), ctypes.byref(lat),
                                       float(timeout_s)), "server_wait")
        return list(res), lat.value

    def replay(self, offsets_s, ref_ids, host_frames, box: int = 5, phases: bool = False):
        """Open-loop replay; returns (latencies, results) and, with phases,
        also each request's (late, queued, issuing, device + completion,
        device time, its copy part) seconds."""
        n = len(offsets_s)
        offs = (ctypes.c_double * n)(*[float(x) for x in offsets_s])
        refs = (_ip * n)(*[int(x) for x in ref_ids])
        frames = (_vp * n)(*[int(x) for x in host_frames])
        lat = (ctypes.c_double * n)()
        res = (ctypes.c_double * (5 * n))()
        ph = (ctypes.c_double * (6 * n))()
        check(lib().glsfft_server_replay_traced(self.handle, n, ctypes.cast(offs, _dp), refs,
                                                frames, int(box), ctypes.cast(lat, _dp),
                                                ctypes.cast(res, _dp), ctypes.cast(ph, _dp)),
              "server_replay")
        out = (list(lat), [list(res[5 * k:5 * k + 5]) for k in range(n)])
        if phases:
            return out + ([list(ph[6 * k:6 * k + 6]) for k in range(n)],)
        return out

    def set_frame_read(self, direct: bool) -> None:
        """True (the default): the row kernel reads page-locked host frames
        itself (no copy-engine transfer); False: a copy-engine transfer."""
        check(lib().glsfft_server_set_frame_read(self.handle, int(bool(direct))),
              "server_set_frame_read")

    def stats(self) -> dict:
        out = (ctypes.c_longlong * 8)()
        check(lib().glsfft_server_stats(self.handle, out), "server_stats")
        return dict(zip(self.STATS, list(out)))

    def close(self) -> None:
        if self.handle:
            lib().glsfft_server_destroy(self.handle)
            self.handle = _vp()

    def __enter__(self):
        return self

    def __exit__(self, *exc):
        self.close()

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass
