"""In-tree build of libsphnj.so (CUDA for sm_103a + host C++).

Each translation unit is compiled by its own nvcc process, in parallel, with a
single -gencode for sm_103a, then linked into sphnj_gb300/_lib/libsphnj.so.
Objects go to sphnj_gb300/_build/.  A unit is recompiled only when it or a
header is newer than its object.
"""
from __future__ import annotations

import concurrent.futures as cf
import os
import shutil
import subprocess
from pathlib import Path

PKG = Path(__file__).resolve().parent
ROOT = PKG.parent
CSRC = PKG / "csrc"
BUILD = PKG / "_build"
LIBDIR = PKG / "_lib"
LIB = LIBDIR / "libsphnj.so"

ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]
NVCC_FLAGS = ["-O3", "-std=c++17", "-lineinfo", "-Xcompiler", "-fPIC", "-Xptxas", "-O3",
              "--expt-relaxed-constexpr", f"-I{ROOT / 'include'}"]


def nvcc() -> str:
    for cand in (os.environ.get("NVCC"), shutil.which("nvcc"), "/usr/local/cuda/bin/nvcc"):
        if cand and Path(cand).exists():
            return cand
    raise RuntimeError("nvcc not found")


def _sources() -> list[Path]:
    return sorted(list(CSRC.glob("*.cu")) + list(CSRC.glob("*.cpp")))


def _headers() -> list[Path]:
    return sorted(list(CSRC.glob("*.h")) + list(CSRC.glob("*.cuh")) + list((ROOT / "include").glob("*.h")))


def _compile(src: Path, verbose: bool) -> Path:
    obj = BUILD / (src.name + ".o")
    newest_dep = max([src.stat().st_mtime] + [h.stat().st_mtime for h in _headers()])
    if obj.exists() and obj.stat().st_mtime >= newest_dep:
        return obj
    if src.suffix == ".cu":
        cmd = [nvcc(), *ARCH, *NVCC_FLAGS, "-c", str(src), "-o", str(obj)]
    else:
        cmd = [nvcc(), "-x", "c++", *NVCC_FLAGS, "-c", str(src), "-o", str(obj)]
    if verbose:
        print(" ".join(cmd), flush=True)
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError(f"compile failed: {src.name}\n{r.stdout}\n{r.stderr}")
    if verbose and (r.stdout or r.stderr):
        print(r.stdout, r.stderr, flush=True)
    return obj


DRIVER_SRC = PKG / "driver" / "sphnj_run.cpp"
DRIVER = LIBDIR / "sphnj_run"


def _build_driver(verbose: bool) -> Path:
    """The host driver executable, linked against libsphnj.so (found next to
    it at run time)."""
    newest = max(DRIVER_SRC.stat().st_mtime, LIB.stat().st_mtime, (ROOT / "include" / "sphnj.h").stat().st_mtime)
    if DRIVER.exists() and DRIVER.stat().st_mtime >= newest:
        return DRIVER
    cxx = os.environ.get("CXX") or shutil.which("g++") or "g++"
    cmd = [cxx, "-O2", "-std=c++17", f"-I{ROOT / 'include'}", str(DRIVER_SRC), f"-L{LIBDIR}", "-lsphnj",
           "-Wl,-rpath,$ORIGIN", "-lpthread", "-o", str(DRIVER)]
    if verbose:
        print(" ".join(cmd), flush=True)
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError(f"driver build failed\n{r.stdout}\n{r.stderr}")
    return DRIVER


def build(verbose: bool = False, jobs: int | None = None) -> Path:
    """Compile and link libsphnj.so and the sphnj_run driver; returns the
    library's path."""
    BUILD.mkdir(exist_ok=True)
    LIBDIR.mkdir(exist_ok=True)
    srcs = _sources()
    with cf.ThreadPoolExecutor(max_workers=jobs or min(8, len(srcs))) as ex:
        objs = list(ex.map(lambda s: _compile(s, verbose), srcs))
    if not (LIB.exists() and LIB.stat().st_mtime >= max(o.stat().st_mtime for o in objs)):
        cmd = [nvcc(), *ARCH, "-shared", "-o", str(LIB), *map(str, objs), "-lcudart_static", "-lrt", "-ldl",
               "-lpthread"]
        if verbose:
            print(" ".join(cmd), flush=True)
        r = subprocess.run(cmd, capture_output=True, text=True)
        if r.returncode != 0:
            raise RuntimeError(f"link failed\n{r.stdout}\n{r.stderr}")
    _build_driver(verbose)
    return LIB


if __name__ == "__main__":
    print(build(verbose=True))
