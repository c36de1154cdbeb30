"""ORACLE - test infrastructure only (the checker and the CPU baseline).

CPU restatement of SPHNJ's particle-step hot path in oracle/sph_oracle.cpp,
built into oracle/_build/liboracle.so and driven through the same ABI shape
as libsphnj (upload / step / download / debug_cells).  Only tests/,
__graft_entry__.smoke() and the CPU-baseline legs of bench.py use it; the
product package sphnj_gb300 never imports it.

Parity pin: state dumps of the reference's own CUDA build, produced by the
harness under oracle/ref/ and committed as tests/golden/ fixtures.
"""
from __future__ import annotations

import ctypes as C
import os
import shutil
import subprocess
from pathlib import Path

import numpy as np

from sphnj_gb300 import abi
from sphnj_gb300.abi import Params, alloc_state, state_struct

HERE = Path(__file__).resolve().parent
SRC = HERE / "sph_oracle.cpp"
LIB_PATH = HERE / "_build" / "liboracle.so"

REFERENCE_PRECISION = 0
FP64 = 1

_lib = None


def build(verbose: bool = False) -> Path:
    """Compiles liboracle.so with g++ (OpenMP, no FP contraction so that x86-64
    and aarch64 hosts give identical results)."""
    LIB_PATH.parent.mkdir(exist_ok=True)
    deps = [SRC, HERE.parent / "include" / "sphnj.h"]
    if LIB_PATH.exists() and LIB_PATH.stat().st_mtime >= max(d.stat().st_mtime for d in deps):
        return LIB_PATH
    cxx = os.environ.get("CXX") or shutil.which("g++") or "g++"
    cmd = [cxx, "-std=c++17", "-O3", "-fPIC", "-shared", "-fopenmp", "-ffp-contract=off",
           f"-I{HERE.parent / 'include'}", str(SRC), "-o", str(LIB_PATH)]
    if verbose:
        print(" ".join(cmd), flush=True)
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError(f"oracle build failed\n{r.stdout}\n{r.stderr}")
    return LIB_PATH


def lib() -> C.CDLL:
    global _lib
    if _lib is None:
        if not LIB_PATH.exists():
            build()
        L = C.CDLL(str(LIB_PATH))
        abi.declare(L, "oracle")
        _lib = L
    return _lib


def max_threads() -> int:
    return lib().oracle_max_threads()


def set_threads(n: int) -> int:
    """OpenMP threads of later oracle steps (n <= 0 keeps the current
    number); returns the number in use."""
    return lib().oracle_set_threads(int(n))


def params_for(case) -> Params:
    """Parameters of a sphnj_gb300.cases.Case derived by the oracle itself
    from the case's input.ini text and particle counts (the reference's
    Parameter::readParameter and initiate restated in oracle/sph_oracle.cpp),
    without the product library."""
    p = Params()
    counts = (C.c_int32 * 4)(case.n_liquid, case.n_gas, case.n_solid, case.n_virt)
    rc = lib().oracle_params_from_ini(case.ini_text().encode(), counts, C.byref(p))
    if rc:
        raise OracleError(f"oracle_params_from_ini: {abi.ERROR_NAMES.get(rc, rc)}")
    return p


class OracleError(RuntimeError):
    pass


class OracleSim:
    """CPU restatement with the Simulation interface of sphnj_gb300."""

    def __init__(self, params: Params, precision: int = REFERENCE_PRECISION, threads: int = 0):
        self.params = params.copy()
        self._lib = lib()
        h = C.c_void_p()
        rc = self._lib.oracle_create(C.byref(self.params), precision, threads, C.byref(h))
        if rc:
            raise OracleError(f"oracle_create: {rc}")
        self._h = h

    def close(self):
        if getattr(self, "_h", None):
            self._lib.oracle_destroy(self._h)
            self._h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def _check(self, rc, what):
        if rc:
            raise OracleError(f"{what}: {abi.ERROR_NAMES.get(rc, rc)}")

    def upload(self, arrays: dict):
        s = state_struct(arrays)
        self._check(self._lib.oracle_upload(self._h, C.byref(s)), "upload")

    def step(self, n: int = 1):
        self._check(self._lib.oracle_step(self._h, int(n)), "step")

    def synchronize(self):
        self._check(self._lib.oracle_error(self._h), "state")

    @property
    def error(self) -> int:
        return self._lib.oracle_error(self._h)

    def download(self, mask: int = abi.F_ALL, into: dict | None = None) -> dict:
        arrays = into if into is not None else alloc_state(self.params)
        s = state_struct(arrays)
        self._check(self._lib.oracle_download(self._h, mask, C.byref(s)), "download")
        return arrays

    def cells(self, kind: int):
        Cn = self.params.cell_number_total
        n = [self.params.fluid_number_total, self.params.solid_number, self.params.virt_number][kind]
        start = np.zeros(Cn, np.int32)
        count = np.zeros(Cn, np.int32)
        lst = np.zeros(max(n, 1) + abi.CELL_SIZE, np.int32)
        nl = C.c_int32()
        PI = abi.PI
        self._check(self._lib.oracle_debug_cells(self._h, kind, start.ctypes.data_as(PI), count.ctypes.data_as(PI),
                                                 lst.ctypes.data_as(PI), C.byref(nl)), "debug_cells")
        return start, count, lst[: nl.value].copy()

    def set_cells(self, fluid=None, solid=None, virt=None):
        args, keep = abi.set_cells_args([fluid, solid, virt])
        self._check(self._lib.oracle_debug_set_cells(self._h, *args), "set_cells")
        del keep

    def set_step(self, step: int):
        self._check(self._lib.oracle_debug_set_step(self._h, int(step)), "set_step")

    def max_speed(self) -> float:
        v = C.c_float()
        self._check(self._lib.oracle_debug_max_speed(self._h, C.byref(v)), "max_speed")
        return v.value

    @property
    def step_index(self) -> int:
        v = C.c_int32()
        self._lib.oracle_get_step(self._h, C.byref(v))
        return v.value
