"""C-ABI checks that need no GPU: the library loads, exports every symbol the
public headers declare, and rejects bad arguments on the host before any
CUDA call (the reference asserts the same conditions, glsFft.cpp:676-681,
glsPhaseCorrelate.cpp:144-150)."""
from __future__ import annotations

import ctypes
import re

import pytest

import glscv_gb300 as g

OK, INVALID, NOT_POW2, SIZE, MISALIGNED = 0, 1, 2, 3, 4
FAKE = 0x10000  # aligned dummy address: never dereferenced, checks fail first


def declared_symbols():
    names = set()
    for h in g.HEADER_PATHS:
        text = h.read_text()
        for m in re.finditer(r"GLSFFT_API\s+[\w\s\*]+?\b(\w+)\s*\(", text):
            names.add(m.group(1))
    return sorted(names)


def test_headers_declare_entry_points():
    names = declared_symbols()
    assert "glsfft_fft2d_c2c" in names and "glsfft_phase_correlate" in names
    assert len(names) >= 10


def test_library_exports_every_declared_symbol(native):
    missing = [n for n in declared_symbols() if not hasattr(native, n)]
    assert not missing, missing


def test_status_strings(native):
    for st in range(0, 10):
        s = native.glsfft_status_string(st)
        assert s and s != b"unknown status"
    assert native.glsfft_status_string(999) == b"unknown status"
    assert native.glsfft_version() >= 100


@pytest.mark.parametrize("rows,cols,flags,expect", [
    (3, 4, 0, NOT_POW2), (4, 6, 0, NOT_POW2), (0, 4, 0, SIZE), (4, 8192, 0, SIZE),
    (-2, 4, 0, SIZE), (4, 4, 4, INVALID), (4, 4, 128, INVALID), (16, 16, 0, INVALID),
])
def test_fft_argument_checks(native, rows, cols, flags, expect):
    # valid arguments with a NULL context end at INVALID (no CUDA call made)
    assert native.glsfft_fft2d_c2c(None, FAKE, FAKE, rows, cols, flags, None) == expect
    assert native.glsfft_fft2d_r2c_promote(None, FAKE, FAKE, rows, cols, flags, None) == expect


def test_fft_pointer_checks(native):
    assert native.glsfft_fft2d_c2c(None, None, FAKE, 4, 4, 0, None) == INVALID
    assert native.glsfft_fft2d_c2c(None, FAKE, None, 4, 4, 0, None) == INVALID
    assert native.glsfft_fft2d_c2c(None, FAKE + 4, FAKE, 4, 4, 0, None) == MISALIGNED
    assert native.glsfft_fft2d_c2c(None, FAKE, FAKE + 4, 4, 4, 0, None) == MISALIGNED
    # CV_32FC1 input needs only 4-byte alignment
    assert native.glsfft_fft2d_r2c_promote(None, FAKE + 4, FAKE, 4, 4, 0, None) == INVALID


def test_phase_correlate_argument_checks(native):
    dx, dy = ctypes.c_double(), ctypes.c_double()
    pc = native.glsfft_phase_correlate
    assert pc(None, FAKE, FAKE, None, 8, 8, 5, ctypes.byref(dx), ctypes.byref(dy), None, None) == INVALID
    assert pc(None, FAKE, FAKE, None, 8, 12, 5, ctypes.byref(dx), ctypes.byref(dy), None, None) == NOT_POW2
    assert pc(None, FAKE, FAKE, None, 8, 8, 0, ctypes.byref(dx), ctypes.byref(dy), None, None) == INVALID
    assert pc(None, FAKE + 2, FAKE, None, 8, 8, 5, ctypes.byref(dx), ctypes.byref(dy), None, None) == MISALIGNED
    assert pc(None, FAKE, FAKE, None, 8, 8, 5, None, ctypes.byref(dy), None, None) == INVALID
    pa = native.glsfft_phase_correlate_async
    assert pa(None, FAKE, FAKE, None, 8, 8, 5, None, None) == INVALID
    assert pa(None, FAKE, FAKE, None, 8, 8, 5, FAKE + 4, None) == INVALID  # NULL ctx after checks


def test_context_calls_reject_null(native):
    assert native.glsfft_context_create(None, 0) == INVALID
    assert native.glsfft_context_destroy(None) == INVALID
    assert native.glsfft_context_set_budget(None, 0) == INVALID
    b = ctypes.c_size_t()
    assert native.glsfft_context_workspace(None, ctypes.byref(b)) == INVALID
    assert native.glsfft_device_status(None, 0) == INVALID
    assert native.glsfft_context_inject_stall(None, 0) == INVALID
    assert native.glsfft_fft2d_reference(None, None, None, 1, 16, 16, 0, 0, None) == INVALID
    assert native.glsfft_phase_correlate_reference(None, None, None, None, 16, 16, 5, 0,
                                                   None, None, None, None) == INVALID


def test_context_create_without_gpu_fails_cleanly(native):
    import torch
    if torch.cuda.is_available():
        pytest.skip("a GPU is present")
    h = ctypes.c_void_p()
    assert native.glsfft_context_create(ctypes.byref(h), 0) != OK
    assert not h.value


def test_python_binding_raises_without_device():
    import torch
    if torch.cuda.is_available():
        pytest.skip("a GPU is present")
    with pytest.raises(g.GlsError):
        g.Context(0)


def test_host_pipeline_and_schedule_calls_reject_bad_arguments(native):
    fl = (ctypes.c_int * 2)(0, 3)
    assert native.glsfft_fft2d_host(None, FAKE, FAKE, 4, 64, 64, 2, fl, 0, None) == INVALID
    assert native.glsfft_fft2d_host(None, None, FAKE, 4, 64, 64, 2, fl, 0, None) == INVALID
    assert native.glsfft_fft2d_host(None, FAKE, FAKE, 0, 64, 64, 2, fl, 0, None) == INVALID
    assert native.glsfft_set_fft_schedule(None, 64, 64, 0, 0) == INVALID
    assert native.glsfft_autotune_fft2d(None, 64, 64, 1, None, None, None, None) == INVALID
    assert native.glsfft_batch_autotune(None, None, 5, None, None, None) == INVALID
    assert native.glsfft_schedule_available(1024, 0, 0) == 1
    assert native.glsfft_schedule_available(1024, 7, 0) == 0
    assert native.glsfft_schedule_available(1024, 6, 0) == 0
    assert native.glsfft_schedule_available(4096, 6, 1) == 1
    assert native.glsfft_schedule_available(4096, 6, 0) == 0
    assert native.glsfft_schedule_available(1000, 0, 0) == 0
    assert native.glsfft_schedule_available(16, 1, 1) == 0
