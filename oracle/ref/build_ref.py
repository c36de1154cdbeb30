"""Builds and runs the SPHNJ reference's own CUDA implementation - test
infrastructure (golden-fixture generation and the reference's GPU timing).

Recipe (no cmake, no reference build system):
  nvcc -rdc=true -gencode arch=compute_103a,code=sm_103a -use_fast_math
       -Xptxas -O3,-dlcm=cg   (the reference's CMakeLists.txt:15-19 flags,
       retargeted from sm_90)
  include path: oracle/ref/shim (windows.h, memory_copy.cuh stand-ins),
                oracle/ref/eigen (Eigen-subset "Eigen/Dense"), then the
                reference's include/.
  sources:      the reference's src/*.cu and src/*.cpp except main.cu (the
                .cpp files are compiled as CUDA, as they include CUDA headers
                indirectly), plus oracle/ref/harness.cu.
Outputs go only to oracle/_ref/ (git-ignored).  The reference tree exists only
in the development container; `stage` copies the source files the recipe
needs into oracle/_ref/src/ (git-ignored, never committed) so that the GPU
machine, which has no reference tree, can build the same binary there.

    python oracle/ref/build_ref.py stage          # development container
    python oracle/ref/build_ref.py build          # anywhere with the sources
    python oracle/ref/build_ref.py run <case_dir> dump 200 1,2,51,52 out/prefix
"""
from __future__ import annotations

import concurrent.futures as cf
import os
import shutil
import subprocess
import sys
from pathlib import Path

HERE = Path(__file__).resolve().parent
OUT = HERE.parent / "_ref"
STAGED = OUT / "src"
# the reference checkout: SPHNJ_REFERENCE, else where the development
# container mounts it
REFERENCE = Path(os.environ.get("SPHNJ_REFERENCE", "/root/reference"))
BIN = OUT / "harness"

FLAGS = ["-std=c++17", "-rdc=true", "-gencode", "arch=compute_103a,code=sm_103a", "-O3", "-use_fast_math",
         "-Xptxas", "-O3,-dlcm=cg", "-w"]


def reference_present() -> bool:
    """True where the reference tree itself is readable (the development
    container), so that build() compiles the harness from it."""
    return (REFERENCE / "src" / "fluid.cu").exists()


def source_root() -> Path:
    if (REFERENCE / "src" / "fluid.cu").exists():
        return REFERENCE
    if (STAGED / "src" / "fluid.cu").exists():
        return STAGED
    raise FileNotFoundError("reference sources not found (run `stage` in the development container)")


def stage() -> Path:
    """Copies the reference's src/ and include/ files into oracle/_ref/src."""
    if not (REFERENCE / "src").exists():
        raise FileNotFoundError(REFERENCE)
    for sub in ("src", "include"):
        d = STAGED / sub
        d.mkdir(parents=True, exist_ok=True)
        for f in sorted((REFERENCE / sub).iterdir()):
            if f.is_file() and f.suffix in (".cu", ".cpp", ".h", ".cuh"):
                shutil.copy2(f, d / f.name)
    return STAGED


def _units(root: Path) -> list[Path]:
    srcs = [p for p in sorted((root / "src").iterdir()) if p.suffix in (".cu", ".cpp") and p.name != "main.cu"]
    return srcs + [HERE / "harness.cu"]


def build(verbose: bool = False) -> Path:
    root = source_root()
    objdir = OUT / "obj"
    objdir.mkdir(parents=True, exist_ok=True)
    inc = [f"-I{HERE / 'shim'}", f"-I{HERE / 'eigen'}", f"-I{root / 'include'}"]
    nvcc = shutil.which("nvcc") or "/usr/local/cuda/bin/nvcc"

    def one(src: Path) -> Path:
        obj = objdir / (src.name + ".o")
        if obj.exists() and obj.stat().st_mtime >= src.stat().st_mtime and obj.stat().st_mtime >= max(
                p.stat().st_mtime for p in list((HERE / "shim").iterdir()) + [HERE / "eigen" / "Eigen" / "Dense"]):
            return obj
        cmd = [nvcc, *FLAGS, *inc, "-x", "cu", "-c", str(src), "-o", str(obj)]
        if verbose:
            print(" ".join(cmd), flush=True)
        r = subprocess.run(cmd, capture_output=True, text=True)
        if r.returncode:
            raise RuntimeError(f"{src.name}:\n{r.stdout}\n{r.stderr}")
        return obj

    with cf.ThreadPoolExecutor(max_workers=min(16, os.cpu_count() or 4)) as ex:
        objs = list(ex.map(one, _units(root)))
    cmd = [nvcc, *FLAGS, *map(str, objs), "-o", str(BIN)]
    if verbose:
        print(" ".join(cmd), flush=True)
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode:
        raise RuntimeError(f"link:\n{r.stdout}\n{r.stderr}")
    return BIN


def prepare_run_dir(case_dir: Path, run_dir: Path) -> Path:
    """The reference opens "..\\\\..\\\\config\\\\input.ini" and
    "..\\\\..\\\\data\\\\*.dat" (parameter.cpp:39,57; sim.cu:44); on Linux those are
    single file names containing backslashes, created here in run_dir."""
    run_dir.mkdir(parents=True, exist_ok=True)
    shutil.copy2(case_dir / "config" / "input.ini", run_dir / "..\\..\\config\\input.ini")
    for f in ("fluid_particle.dat", "solid_particle.dat", "virt_particle.dat"):
        shutil.copy2(case_dir / "data" / f, run_dir / f"..\\..\\data\\{f}")
    return run_dir


def run(case_dir, args: list[str], run_dir=None, timeout=None) -> subprocess.CompletedProcess:
    case_dir = Path(case_dir).resolve()
    run_dir = Path(run_dir or (OUT / "run" / case_dir.name)).resolve()
    prepare_run_dir(case_dir, run_dir)
    return subprocess.run([str(BIN), *args], cwd=run_dir, capture_output=True, text=True, timeout=timeout)


if __name__ == "__main__":
    cmd = sys.argv[1] if len(sys.argv) > 1 else "build"
    if cmd == "stage":
        print(stage())
    elif cmd == "build":
        print(build(verbose="-v" in sys.argv))
    elif cmd == "run":
        r = run(sys.argv[2], sys.argv[3:])
        sys.stdout.write(r.stdout)
        sys.stderr.write(r.stderr)
        sys.exit(r.returncode)
