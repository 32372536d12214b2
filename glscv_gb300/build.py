"""Build recipe for the native library ``glscv_gb300/lib/libglscv_gb300.so``.

Every CUDA translation unit is compiled by nvcc for sm_103a only
(``-gencode arch=compute_103a,code=sm_103a -lineinfo``), host C++ units by
nvcc's host pass, in parallel, into ``glscv_gb300/_build``; then one shared
library is linked in-tree (static CUDA runtime, so the library needs nothing
from PyTorch).  Objects are rebuilt when their source, any header, or the
flags change.  Run as ``python -m glscv_gb300.build``.
"""
from __future__ import annotations

import hashlib
import os
import subprocess
import sys
from concurrent.futures import ThreadPoolExecutor
from pathlib import Path

PKG = Path(__file__).resolve().parent
ROOT = PKG.parent
CSRC = PKG / "csrc"
INCLUDE = ROOT / "include"
BUILD = PKG / "_build"
LIB_DIR = PKG / "lib"
LIB = LIB_DIR / "libglscv_gb300.so"

ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]
COMMON = ["-O3", "-std=c++17", "-lineinfo", "-Xcompiler", "-fPIC,-fvisibility=hidden",
          f"-I{INCLUDE}", f"-I{CSRC}"]
CU_FLAGS = ARCH + COMMON + ["-Xptxas", "-warn-spills"]
CPP_FLAGS = COMMON


def nvcc() -> str:
    for cand in (os.environ.get("NVCC"), "/usr/local/cuda/bin/nvcc", "nvcc"):
        if cand and (os.path.sep not in cand or Path(cand).exists()):
            return cand
    return "nvcc"


def sources() -> list[Path]:
    return sorted(list(CSRC.glob("*.cu")) + list(CSRC.glob("*.cpp")))


def _headers_stamp() -> str:
    h = hashlib.sha256()
    for p in sorted(list(CSRC.glob("*.h")) + list(CSRC.glob("*.cuh")) + list(INCLUDE.rglob("*.h"))):
        h.update(p.name.encode())
        h.update(p.read_bytes())
    return h.hexdigest()


def _obj_for(src: Path) -> Path:
    return BUILD / (src.name + ".o")


def _stamp_for(src: Path, flags: list[str], hstamp: str) -> str:
    h = hashlib.sha256()
    h.update(src.read_bytes())
    h.update(" ".join(flags).encode())
    h.update(hstamp.encode())
    return h.hexdigest()


def _compile(src: Path, flags: list[str], hstamp: str, verbose: bool) -> tuple[Path, bool]:
    obj = _obj_for(src)
    stamp_file = obj.with_suffix(".stamp")
    stamp = _stamp_for(src, flags, hstamp)
    if obj.exists() and stamp_file.exists() and stamp_file.read_text() == stamp:
        return obj, False
    cmd = [nvcc()] + flags + ["-c", str(src), "-o", str(obj)]
    if verbose:
        print(" ".join(cmd), flush=True)
    res = subprocess.run(cmd, capture_output=True, text=True)
    if res.returncode != 0:
        raise RuntimeError(f"nvcc failed for {src.name}:\n{res.stdout}\n{res.stderr}")
    if verbose and res.stderr.strip():
        print(res.stderr, file=sys.stderr)
    stamp_file.write_text(stamp)
    return obj, True


def build(verbose: bool = False, jobs: int | None = None) -> Path:
    BUILD.mkdir(exist_ok=True)
    LIB_DIR.mkdir(exist_ok=True)
    hstamp = _headers_stamp()
    srcs = sources()
    jobs = jobs or min(len(srcs), os.cpu_count() or 4)
    with ThreadPoolExecutor(max_workers=jobs) as ex:
        futs = [ex.submit(_compile, s, CU_FLAGS if s.suffix == ".cu" else CPP_FLAGS, hstamp, verbose)
                for s in srcs]
        results = [f.result() for f in futs]
    objs = [o for o, _ in results]
    rebuilt = any(r for _, r in results)
    if rebuilt or not LIB.exists() or any(o.stat().st_mtime > LIB.stat().st_mtime for o in objs):
        tmp = LIB.with_suffix(".so.tmp")
        cmd = [nvcc()] + ARCH + ["-shared", "-o", str(tmp)] + [str(o) for o in objs] + ["-lpthread"]
        if verbose:
            print(" ".join(cmd), flush=True)
        res = subprocess.run(cmd, capture_output=True, text=True)
        if res.returncode != 0:
            raise RuntimeError(f"link failed:\n{res.stdout}\n{res.stderr}")
        os.replace(tmp, LIB)
    return LIB


if __name__ == "__main__":
    print(build(verbose="-v" in sys.argv))
