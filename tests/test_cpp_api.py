"""The C++ drop-in layer (include/gls/glsCV.h): the test program in
tests/cpp/test_gls_api.cpp is compiled against the public headers and linked
to the native library with the host compiler alone (no CUDA headers needed by
a caller) -- a CPU check -- and run on the GPU."""
from __future__ import annotations

import subprocess
from pathlib import Path

import pytest

ROOT = Path(__file__).resolve().parents[1]
SRC = ROOT / "tests" / "cpp" / "test_gls_api.cpp"


def _build(native, tmp_path_factory) -> Path:
    import glscv_gb300
    out = tmp_path_factory.mktemp("cpp") / "test_gls_api"
    lib_dir = glscv_gb300.LIB_PATH.parent
    cmd = ["g++", "-std=c++17", "-O1", "-Wall", f"-I{ROOT / 'include'}", str(SRC), "-o", str(out),
           f"-L{lib_dir}", "-lglscv_gb300", f"-Wl,-rpath,{lib_dir}"]
    res = subprocess.run(cmd, capture_output=True, text=True)
    assert res.returncode == 0, res.stderr
    return out


@pytest.fixture(scope="module")
def cpp_binary(native, tmp_path_factory):
    return _build(native, tmp_path_factory)


def test_cpp_api_compiles_and_links(cpp_binary):
    assert cpp_binary.exists()


@pytest.mark.gpu
def test_cpp_api_runs(cpp_binary, torch_cuda):
    res = subprocess.run([str(cpp_binary)], capture_output=True, text=True, timeout=300)
    assert res.returncode == 0, res.stdout + res.stderr
    assert "ALL OK" in res.stdout


def test_arena_allocator_host_unit(tmp_path):
    """The serving loop's device-memory arena, compiled without CUDA."""
    src = ROOT / "tests" / "cpp" / "test_arena.cpp"
    out = tmp_path / "test_arena"
    res = subprocess.run(["g++", "-std=c++17", "-O1", "-Wall",
                          f"-I{ROOT / 'glscv_gb300' / 'csrc'}", str(src), "-o", str(out)],
                         capture_output=True, text=True)
    assert res.returncode == 0, res.stderr
    run = subprocess.run([str(out)], capture_output=True, text=True, timeout=60)
    assert run.returncode == 0 and "ALL OK" in run.stdout, run.stdout


def test_plan_cache_host_unit(tmp_path):
    """The autotuner's plan cache file format and lookup, compiled without CUDA."""
    src = ROOT / "tests" / "cpp" / "test_plan_cache.cpp"
    out = tmp_path / "test_plan_cache"
    res = subprocess.run(["g++", "-std=c++17", "-O1", "-Wall",
                          f"-I{ROOT / 'glscv_gb300' / 'csrc'}", str(src), "-o", str(out)],
                         capture_output=True, text=True)
    assert res.returncode == 0, res.stderr
    run = subprocess.run([str(out), str(tmp_path / "cache.jsonl")], capture_output=True,
                         text=True, timeout=60)
    assert run.returncode == 0 and "ALL OK" in run.stdout, run.stdout


def test_batch_layout_host_unit(tmp_path):
    """The batch plans' column-tiled workspace arithmetic (layout, workspace
    rules, the swizzled stage positions) against emulated tensor boxes,
    compiled without CUDA."""
    src = ROOT / "tests" / "cpp" / "test_batch_layout.cpp"
    out = tmp_path / "test_batch_layout"
    res = subprocess.run(["g++", "-std=c++17", "-O1", "-Wall",
                          f"-I{ROOT / 'glscv_gb300' / 'csrc'}", str(src), "-o", str(out)],
                         capture_output=True, text=True)
    assert res.returncode == 0, res.stderr
    run = subprocess.run([str(out)], capture_output=True, text=True, timeout=60)
    assert run.returncode == 0 and "ALL OK" in run.stdout, run.stdout


def test_batch_order_host_unit(tmp_path):
    """The batch plans' work-list order: every tile listed once, every item
    after all tiles of its image's previous pass (no wait on an unclaimed
    item), over random batches and lags, compiled without CUDA."""
    src = ROOT / "tests" / "cpp" / "test_batch_order.cpp"
    out = tmp_path / "test_batch_order"
    res = subprocess.run(["g++", "-std=c++17", "-O1", "-Wall",
                          f"-I{ROOT / 'glscv_gb300' / 'csrc'}", str(src), "-o", str(out)],
                         capture_output=True, text=True)
    assert res.returncode == 0, res.stderr
    run = subprocess.run([str(out)], capture_output=True, text=True, timeout=120)
    assert run.returncode == 0 and "ALL OK" in run.stdout, run.stdout
