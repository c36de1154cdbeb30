"""sphnj_gb300 - GB300-native particle-step library for SPHNJ cases.

Python host mirror of the C ABI in include/sphnj.h.  The compute path is
libsphnj.so (hand-written sm_103a kernels); this module only loads it, moves
host arrays across the ABI, and reads reference case directories
(config/input.ini + data/*.dat).  There is no CPU fallback: creating a
simulation without the built library or without a CUDA device raises.

Reference seam being replaced: DeviceFunction::GPUCalulation(Sim*)
(include/function.cuh:12, src/calculation.cu:14-18) and the host
initialisation in src/main.cu:14-29.
"""
from __future__ import annotations

import ctypes as C
import os
from pathlib import Path

import numpy as np

from . import abi
from .abi import Params, alloc_state, state_struct

PKG = Path(__file__).resolve().parent
LIB_PATH = PKG / "_lib" / "libsphnj.so"

_lib = None


class SphnjError(RuntimeError):
    def __init__(self, code: int, msg: str = ""):
        self.code = code
        super().__init__(f"{abi.ERROR_NAMES.get(code, code)}: {msg}" if msg else abi.ERROR_NAMES.get(code, str(code)))


def build(verbose: bool = False) -> Path:
    from ._build import build as _b

    return _b(verbose=verbose)


def lib() -> C.CDLL:
    """The loaded libsphnj.so (raises if it has not been built)."""
    global _lib
    if _lib is None:
        if not LIB_PATH.exists():
            raise SphnjError(abi.ERR_NO_DEVICE, f"{LIB_PATH} is missing: run sphnj_gb300.build()")
        L = C.CDLL(str(LIB_PATH))
        abi.declare(L, "sphnj")
        L.sphnj_params_read_ini.argtypes = [C.c_char_p, C.POINTER(Params)]
        L.sphnj_params_read_counts.argtypes = [C.c_char_p, C.POINTER(Params)]
        L.sphnj_params_derive.argtypes = [C.POINTER(Params)]
        L.sphnj_read_particles.argtypes = [C.c_char_p, C.POINTER(Params), C.POINTER(abi.HostState)]
        L.sphnj_abi_sizeof.argtypes = [C.c_int]
        L.sphnj_upload_fields.argtypes = [C.c_void_p, C.c_uint32, C.POINTER(abi.HostState)]
        L.sphnj_upload_fields.restype = C.c_int
        L.sphnj_step_exchange.argtypes = [C.c_void_p, C.c_int, C.c_uint32, C.POINTER(abi.HostState), C.c_uint32,
                                          C.POINTER(abi.HostState)]
        L.sphnj_step_exchange.restype = C.c_int
        L.sphnj_profile_stage_count.argtypes = []
        L.sphnj_profile_stage_count.restype = C.c_int
        L.sphnj_profile_stage_name.argtypes = [C.c_int]
        L.sphnj_profile_stage_name.restype = C.c_char_p
        L.sphnj_profile_enable.argtypes = [C.c_void_p, C.c_int]
        L.sphnj_profile_enable.restype = C.c_int
        L.sphnj_profile_read.argtypes = [C.c_void_p, C.POINTER(C.c_double), C.POINTER(C.c_int64),
                                         C.POINTER(C.c_int64)]
        L.sphnj_profile_read.restype = C.c_int
        L.sphnj_stat_launches.argtypes = [C.c_void_p, C.POINTER(C.c_uint64)]
        L.sphnj_stat_launches.restype = C.c_int
        L.sphnj_set_tiling.argtypes = [C.c_void_p, C.c_int, C.c_int]
        L.sphnj_set_tiling.restype = C.c_int
        L.sphnj_set_graphs.argtypes = [C.c_void_p, C.c_int]
        L.sphnj_set_graphs.restype = C.c_int
        for f in ("sphnj_params_read_ini", "sphnj_params_read_counts", "sphnj_params_derive",
                  "sphnj_read_particles", "sphnj_abi_sizeof"):
            getattr(L, f).restype = C.c_int
        if (L.sphnj_abi_sizeof(0) != C.sizeof(Params) or L.sphnj_abi_sizeof(1) != C.sizeof(abi.HostState)
                or L.sphnj_abi_sizeof(2) != C.sizeof(abi.Diag) or L.sphnj_abi_sizeof(3) != C.sizeof(abi.Tuning)):
            raise SphnjError(abi.ERR_ARG, "ABI layout mismatch between include/sphnj.h and sphnj_gb300/abi.py")
        _lib = L
    return _lib


# ---- host-side configuration and case I/O (no GPU needed) -------------------

def read_ini(path) -> tuple[Params, int]:
    """Reads an input.ini with the reference's Config semantics.  Returns the
    params and the status (ERR_CONFIG when the reference would refuse it)."""
    p = Params()
    rc = lib().sphnj_params_read_ini(str(path).encode(), C.byref(p))
    if rc not in (abi.OK, abi.ERR_CONFIG):
        raise SphnjError(rc, str(path))
    return p, rc


def derive(p: Params) -> Params:
    rc = lib().sphnj_params_derive(C.byref(p))
    if rc:
        raise SphnjError(rc, "derive")
    return p


def read_counts(data_dir, p: Params) -> Params:
    rc = lib().sphnj_params_read_counts(str(data_dir).encode(), C.byref(p))
    if rc:
        raise SphnjError(rc, str(data_dir))
    return p


def read_particles(data_dir, p: Params) -> dict:
    arrays = alloc_state(p, abi.INPUT_FIELDS)
    s = state_struct(arrays)
    rc = lib().sphnj_read_particles(str(data_dir).encode(), C.byref(p), C.byref(s))
    if rc:
        raise SphnjError(rc, str(data_dir))
    return arrays


def load_case(case_dir) -> tuple[Params, dict]:
    """Reads <case_dir>/config/input.ini and <case_dir>/data/*.dat in the
    order of Parameter::initiate (parameter.h:28-33): particle counts, ini
    keys, derived constants; then the particle files (sim.cu:40-60)."""
    case_dir = Path(case_dir)
    p, rc = read_ini(case_dir / "config" / "input.ini")
    if rc:
        raise SphnjError(rc, "input.ini: a required key is missing or invalid")
    read_counts(case_dir / "data", p)
    derive(p)
    return p, read_particles(case_dir / "data", p)


# ---- simulation context -----------------------------------------------------

class Simulation:
    """One scene on the current CUDA device (libsphnj context)."""

    def __init__(self, params: Params, form: int = abi.FORM_PLAIN):
        self.params = params.copy()
        self._lib = lib()
        h = C.c_void_p()
        rc = self._lib.sphnj_create(C.byref(self.params), form, C.byref(h))
        if rc:
            raise SphnjError(rc, "sphnj_create")
        self._h = h

    def _check(self, rc: int, what: str):
        if rc:
            msg = self._lib.sphnj_last_error(self._h).decode()
            raise SphnjError(rc, f"{what}: {msg}")

    def close(self):
        if getattr(self, "_h", None):
            self._lib.sphnj_destroy(self._h)
            self._h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def __enter__(self):
        return self

    def __exit__(self, *exc):
        self.close()

    def set_stream(self, stream_handle: int | None):
        self._check(self._lib.sphnj_set_stream(self._h, C.c_void_p(stream_handle or 0)), "set_stream")

    def upload(self, arrays: dict):
        s = state_struct(arrays)
        self._check(self._lib.sphnj_upload(self._h, C.byref(s)), "upload")

    def set_tiling(self, tiled: bool = True, tile_h: int = 16):
        self._check(self._lib.sphnj_set_tiling(self._h, 1 if tiled else 0, int(tile_h)), "set_tiling")

    def set_graphs(self, on: bool = True):
        self._check(self._lib.sphnj_set_graphs(self._h, 1 if on else 0), "set_graphs")

    def set_launch_chaining(self, on: bool = True):
        """Programmatic dependent launch between the kernels of a step
        (sphnj_set_launch_chaining)."""
        self._check(self._lib.sphnj_set_launch_chaining(self._h, 1 if on else 0), "set_launch_chaining")

    def set_block_sizes(self, shift_threads: int = 0, pair_threads: int = 0):
        """Threads per block of the tiled shifting passes and pair pass (0: the
        launch kind's default; sphnj_set_block_sizes)."""
        self._check(self._lib.sphnj_set_block_sizes(self._h, int(shift_threads), int(pair_threads)), "block_sizes")

    def block_sizes(self) -> tuple:
        a, b = C.c_int(), C.c_int()
        self._check(self._lib.sphnj_get_block_sizes(self._h, C.byref(a), C.byref(b)), "block_sizes")
        return a.value, b.value

    def set_neighbour_lists(self, on: bool = True):
        self._check(self._lib.sphnj_set_neighbour_lists(self._h, 1 if on else 0), "set_neighbour_lists")

    def sweeps(self) -> dict:
        t, h, l = C.c_int(), C.c_int(), C.c_int()
        self._check(self._lib.sphnj_get_sweeps(self._h, C.byref(t), C.byref(h), C.byref(l)), "get_sweeps")
        return {"tiled": bool(t.value), "tile_h": h.value, "lists": bool(l.value)}

    def autotune(self, steps: int = 5) -> dict:
        """Times the sweep configurations from the current state (which is put
        back) and installs the fastest (sphnj_autotune)."""
        r = abi.Tuning()
        self._check(self._lib.sphnj_autotune(self._h, int(steps), C.byref(r)), "autotune")
        return r.as_dict()

    def upload_fields(self, mask: int, arrays: dict):
        s = state_struct(arrays)
        self._check(self._lib.sphnj_upload_fields(self._h, int(mask), C.byref(s)), "upload_fields")

    def step(self, n: int = 1):
        self._check(self._lib.sphnj_step(self._h, int(n)), "step")

    def step_exchange(self, n: int, in_mask: int, arrays_in: dict | None, out_mask: int,
                      into: dict | None) -> dict | None:
        """upload_fields(in_mask, arrays_in) + step(n) + download(out_mask,
        into) as one call (sphnj_step_exchange), with the host transfers
        overlapped with the steps; returns `into`."""
        sin = state_struct(arrays_in) if arrays_in is not None else None
        sout = state_struct(into) if into is not None else None
        self._check(self._lib.sphnj_step_exchange(self._h, int(n), int(in_mask),
                                                  C.byref(sin) if sin is not None else None, int(out_mask),
                                                  C.byref(sout) if sout is not None else None), "step_exchange")
        return into

    def profile_enable(self, on: bool = True):
        self._check(self._lib.sphnj_profile_enable(self._h, 1 if on else 0), "profile_enable")

    def profile_read(self) -> dict:
        """{stage: (device ms, timed calls, kernels launched)} since enabling."""
        n = self._lib.sphnj_profile_stage_count()
        ms = (C.c_double * n)()
        calls = (C.c_int64 * n)()
        kern = (C.c_int64 * n)()
        self._check(self._lib.sphnj_profile_read(self._h, ms, calls, kern), "profile_read")
        return {self._lib.sphnj_profile_stage_name(i).decode(): (ms[i], calls[i], kern[i]) for i in range(n)}

    def launches(self) -> int:
        v = C.c_uint64()
        self._check(self._lib.sphnj_stat_launches(self._h, C.byref(v)), "stat_launches")
        return v.value

    def synchronize(self):
        self._check(self._lib.sphnj_synchronize(self._h), "synchronize")

    def host_state(self, fields=None) -> dict:
        """Zeroed host arrays for this scene's state (all fields, or those
        named) in pinned, device-mapped memory (sphnj_host_alloc): uploads
        and downloads of the fluid positions, velocities, densities and
        pressures held there run as one kernel over the host link."""
        return alloc_state(self.params, fields, lib=self._lib)

    def download(self, mask: int = abi.F_ALL, into: dict | None = None) -> dict:
        arrays = into if into is not None else alloc_state(self.params)
        s = state_struct(arrays)
        self._check(self._lib.sphnj_download(self._h, mask, C.byref(s)), "download")
        return arrays

    def cells(self, kind: int):
        """(start, count, list) of the current cell lists of one particle kind
        (0 fluid, 1 solid, 2 virtual), in the reference's per-cell order."""
        Cn = self.params.cell_number_total
        n = [self.params.fluid_number_total, self.params.solid_number, self.params.virt_number][kind]
        start = np.zeros(Cn, np.int32)
        count = np.zeros(Cn, np.int32)
        lst = np.zeros(max(n, 1), np.int32)
        nl = C.c_int32()
        PI = abi.PI
        self._check(self._lib.sphnj_debug_cells(self._h, kind, start.ctypes.data_as(PI), count.ctypes.data_as(PI),
                                                lst.ctypes.data_as(PI), C.byref(nl)), "debug_cells")
        return start, count, lst[: nl.value].copy()

    def set_cells(self, fluid=None, solid=None, virt=None):
        """Replaces the current cell lists; each argument is (count[C], list)."""
        args, keep = abi.set_cells_args([fluid, solid, virt])
        self._check(self._lib.sphnj_debug_set_cells(self._h, *args), "set_cells")
        del keep

    def set_step(self, step: int):
        self._check(self._lib.sphnj_debug_set_step(self._h, int(step)), "set_step")

    def diagnostics(self) -> dict:
        """Global diagnostics reduced on the device in FP64 (sphnj_diagnostics)."""
        out = abi.Diag()
        self._check(self._lib.sphnj_diagnostics(self._h, C.byref(out)), "diagnostics")
        return out.as_dict()

    def probe(self, points) -> np.ndarray:
        """Shepard probes at points (n, 2): rows vx, vy, p, rho (sphnj_probe)."""
        pts = np.ascontiguousarray(points, np.float32).reshape(-1, 2)
        out = np.empty((len(pts), 4), np.float32)
        self._check(self._lib.sphnj_probe(self._h, len(pts), pts.ctypes.data_as(abi.PF), out.ctypes.data_as(abi.PF)),
                    "probe")
        return out

    def checkpoint(self) -> np.ndarray:
        """The complete device state as bytes (sphnj_checkpoint_save)."""
        n = C.c_uint64()
        self._check(self._lib.sphnj_checkpoint_size(self._h, C.byref(n)), "checkpoint_size")
        buf = np.empty(n.value, np.uint8)
        self._check(self._lib.sphnj_checkpoint_save(self._h, buf.ctypes.data, n.value), "checkpoint_save")
        return buf

    def restore(self, buf: np.ndarray):
        buf = np.ascontiguousarray(buf, np.uint8)
        self._check(self._lib.sphnj_checkpoint_load(self._h, buf.ctypes.data, buf.nbytes), "checkpoint_load")

    def save(self, path):
        self._check(self._lib.sphnj_checkpoint_write(self._h, str(path).encode()), "checkpoint_write")

    def load(self, path):
        self._check(self._lib.sphnj_checkpoint_read(self._h, str(path).encode()), "checkpoint_read")

    def max_speed(self) -> float:
        v = C.c_float()
        self._check(self._lib.sphnj_debug_max_speed(self._h, C.byref(v)), "max_speed")
        return v.value

    @property
    def step_index(self) -> int:
        v = C.c_int32()
        self._check(self._lib.sphnj_get_step(self._h, C.byref(v)), "get_step")
        return v.value


class Batch:
    """Independent scenes advanced together: every stage of a step is one
    launch over all of them (sphnj_batch_* in include/sphnj.h).  The scenes
    are uploaded Simulations at the same step with the same sort_every_step;
    they stay usable for download (and upload) and must outlive the batch."""

    def __init__(self, sims):
        self.sims = list(sims)
        self._lib = lib()
        handles = (C.c_void_p * len(self.sims))(*[s._h.value for s in self.sims])
        h = C.c_void_p()
        rc = self._lib.sphnj_batch_create(handles, len(self.sims), C.byref(h))
        if rc:
            raise SphnjError(rc, "sphnj_batch_create: scenes must be uploaded, at the same step, share "
                                 "sort_every_step and belong to no other batch")
        self._h = h

    def _check(self, rc: int, what: str):
        if rc:
            raise SphnjError(rc, f"{what}: {self._lib.sphnj_batch_last_error(self._h).decode()}")

    def close(self):
        if getattr(self, "_h", None):
            self._lib.sphnj_batch_destroy(self._h)
            self._h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def __enter__(self):
        return self

    def __exit__(self, *exc):
        self.close()

    def set_stream(self, stream_handle: int | None):
        self._check(self._lib.sphnj_batch_set_stream(self._h, C.c_void_p(stream_handle or 0)), "set_stream")

    def set_tiling(self, tiled: bool = True, tile_h: int = 16):
        self._check(self._lib.sphnj_batch_set_tiling(self._h, 1 if tiled else 0, int(tile_h)), "set_tiling")

    def set_graphs(self, on: bool = True):
        self._check(self._lib.sphnj_batch_set_graphs(self._h, 1 if on else 0), "set_graphs")

    def set_launch_chaining(self, on: bool = True):
        self._check(self._lib.sphnj_batch_set_launch_chaining(self._h, 1 if on else 0), "set_launch_chaining")

    def set_block_sizes(self, shift_threads: int = 0, pair_threads: int = 0):
        self._check(self._lib.sphnj_batch_set_block_sizes(self._h, int(shift_threads), int(pair_threads)),
                    "block_sizes")

    def set_scene_tiling(self, scene: int, tile_h: int, lists: bool = True):
        """One scene's own tile height and list switch (sphnj_batch_set_scene_tiling)."""
        self._check(self._lib.sphnj_batch_set_scene_tiling(self._h, int(scene), int(tile_h), 1 if lists else 0),
                    "scene_tiling")

    def scene_tiling(self, scene: int) -> tuple:
        a, b = C.c_int(), C.c_int()
        self._check(self._lib.sphnj_batch_get_scene_tiling(self._h, int(scene), C.byref(a), C.byref(b)),
                    "scene_tiling")
        return a.value, bool(b.value)

    def set_neighbour_lists(self, on: bool = True):
        self._check(self._lib.sphnj_batch_set_neighbour_lists(self._h, 1 if on else 0), "set_neighbour_lists")

    def sweeps(self) -> dict:
        t, h, l = C.c_int(), C.c_int(), C.c_int()
        self._check(self._lib.sphnj_batch_get_sweeps(self._h, C.byref(t), C.byref(h), C.byref(l)), "get_sweeps")
        return {"tiled": bool(t.value), "tile_h": h.value, "lists": bool(l.value)}

    def autotune(self, steps: int = 5) -> dict:
        r = abi.Tuning()
        self._check(self._lib.sphnj_batch_autotune(self._h, int(steps), C.byref(r)), "autotune")
        return r.as_dict()

    def step(self, n: int = 1):
        self._check(self._lib.sphnj_batch_step(self._h, int(n)), "step")

    def synchronize(self):
        self._check(self._lib.sphnj_batch_synchronize(self._h), "synchronize")

    def profile_enable(self, on: bool = True):
        self._check(self._lib.sphnj_batch_profile_enable(self._h, 1 if on else 0), "profile_enable")

    def profile_read(self) -> dict:
        """{stage: (device ms, timed calls, kernels launched)} since enabling."""
        n = self._lib.sphnj_profile_stage_count()
        ms = (C.c_double * n)()
        calls = (C.c_int64 * n)()
        kern = (C.c_int64 * n)()
        self._check(self._lib.sphnj_batch_profile_read(self._h, ms, calls, kern), "profile_read")
        return {self._lib.sphnj_profile_stage_name(i).decode(): (ms[i], calls[i], kern[i]) for i in range(n)}

    def launches(self) -> int:
        v = C.c_uint64()
        self._check(self._lib.sphnj_batch_stat_launches(self._h, C.byref(v)), "stat_launches")
        return v.value


__all__ = ["abi", "Params", "Simulation", "Batch", "SphnjError", "build", "lib", "load_case", "read_ini", "derive",
           "read_counts", "read_particles", "alloc_state", "state_struct"]
