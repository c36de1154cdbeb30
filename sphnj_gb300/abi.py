"""ctypes mirror of include/sphnj.h (the C ABI of libsphnj).

The structures below must match the header field for field; the library's
``sphnj_abi_sizeof`` is checked against ``ctypes.sizeof`` when the library is
loaded, and the ini-reading tests check field placement through values.
"""
from __future__ import annotations

import ctypes as C

OK = 0
ERR_ARG, ERR_IO, ERR_CONFIG, ERR_COUNT, ERR_CUDA = 1, 2, 3, 4, 5
ERR_CELL_OVERFLOW, ERR_OUT_OF_GRID, ERR_NONFINITE, ERR_WATCHDOG = 6, 7, 8, 9
ERR_UNSUPPORTED, ERR_NO_DEVICE = 10, 11

ERROR_NAMES = {
    0: "ok", 1: "bad argument", 2: "file I/O", 3: "config", 4: "particle count mismatch", 5: "CUDA",
    6: "cell overflow", 7: "particle out of cell grid", 8: "non-finite state", 9: "watchdog",
    10: "unsupported", 11: "no CUDA device",
}

# enumerations (include/types.h:4-67)
LIQUID, GAS = 0, 1
SLIP, NO_SLIP, MOVING = 0, 1, 2
SPLASH, FREE_SURFACE, VICINITY, INNER = 0, 1, 2, 3
NO_PARTICLE, HAS_PARTICLE, HAS_NEAR_PARTICLE = 0, 1, 2
LINEAR_ELASTIC, AUXETIC = 0, 1
HYPER_ELASTIC, PLASTIC = 0, 1
UNCONSTRAINED, FIXED = 0, 1
STRESS_2D, STRAIN_2D = 0, 1
TRANSIENT, STEADY = 0, 1

CELL_SIZE = 64
FORM_PLAIN = 0
FORM_MIXED = 1

F_FLUID_KINEMATICS = 1 << 0
F_FLUID_THERMO = 1 << 1
F_FLUID_FLAGS = 1 << 2
F_FLUID_DERIVED = 1 << 3
F_SOLID_KINEMATICS = 1 << 4
F_SOLID_MATERIAL = 1 << 5
F_SOLID_DERIVED = 1 << 6
F_VIRT = 1 << 7
F_CELL_IDS = 1 << 8
F_ALL = 0x1FF

f32, f64, i32 = C.c_float, C.c_double, C.c_int32


class Params(C.Structure):
    _fields_ = [
        ("gravity", f32 * 2), ("transient_type", i32),
        ("fluid_number", i32 * 2), ("fluid_number_total", i32),
        ("sound_speed", f32 * 2), ("reference_density", f32 * 2), ("reference_density_inverse", f32 * 2),
        ("gamma", f32 * 2), ("viscosity", f32 * 2), ("particle_shift_coef", f32),
        ("gamma_inv", f32 * 2), ("coefficient_p2rho", f32 * 2), ("coefficient_rho2p", f32 * 2),
        ("min_pressure", f32), ("min_density", f32 * 2), ("is_fluid_viscid", i32),
        ("solid_number", i32), ("solid_reference_density", f32), ("youngs_modulus", f32),
        ("poisson_ratio", f32), ("lambda_", f32), ("nu", f32), ("bulk_modulus", f32),
        ("artificial_viscosity", f32 * 2), ("solid_sound_speed", f32), ("fixed_speed", f64 * 2),
        ("constitution_type", i32), ("plastic_type", i32),
        ("auxetic_density", f32), ("auxetic_modulus", f32), ("auxetic_poisson_ratio", f32),
        ("yield_strain", f32), ("yield_stress", f32), ("harden_strain", f32), ("harden_coef", f32),
        ("auxetic_lambda", f32), ("auxetic_nu", f32),
        ("virt_number", i32),
        ("cell_xmin", f32 * 2), ("cell_xmax", f32 * 2), ("domain_xmin", f32 * 2), ("domain_xmax", f32 * 2),
        ("cell_number", i32 * 2), ("interval", f32 * 2), ("interval_inv", f32 * 2), ("cell_number_total", i32),
        ("dt", f32), ("istart", i32), ("iend", i32), ("solid_sub_step", i32), ("shift_per_step", i32),
        ("result_interval", i32), ("sort_every_step", i32),
        ("smoothing_length", f32), ("particle_diameter", f32), ("particle_volume", f32),
        ("diameter_square", f32), ("thread_num", i32), ("smoothing_length_square", f32),
        ("smoothing_length_inverse", f32), ("smoothing_length_inverse_square", f32),
        ("impact_length_hsml_ratio", f32), ("impact_distance_square", f32),
        ("kernel_coefficient_1", f32), ("kernel_coefficient_2", f32), ("kernel_differential", f32),
        ("coefficient_3d_to_2d", f32),
    ]

    def to_dict(self) -> dict:
        out = {}
        for name, typ in self._fields_:
            v = getattr(self, name)
            out[name] = list(v) if hasattr(v, "__len__") else v
        return out

    def copy(self) -> "Params":
        c = Params()
        C.memmove(C.byref(c), C.byref(self), C.sizeof(Params))
        return c


PF, PD, PI = C.POINTER(C.c_float), C.POINTER(C.c_double), C.POINTER(C.c_int32)

# (field, ctype pointer, numpy dtype, per-particle width, kind)
STATE_FIELDS = [
    ("fluid_position", PF, "float32", 2, "fluid"),
    ("fluid_velocity", PF, "float32", 2, "fluid"),
    ("fluid_density", PF, "float32", 1, "fluid"),
    ("fluid_pressure", PF, "float32", 1, "fluid"),
    ("fluid_phase", PI, "int32", 1, "fluid"),
    ("fluid_boundary_type", PI, "int32", 1, "fluid"),
    ("fluid_has_near_particle", PI, "int32", 1, "fluid"),
    ("fluid_du_dx", PF, "float32", 4, "fluid"),
    ("fluid_gradient", PF, "float32", 2, "fluid"),
    ("fluid_du_dt", PF, "float32", 2, "fluid"),
    ("fluid_color", PF, "float32", 1, "fluid"),
    ("fluid_drho_dt", PF, "float32", 1, "fluid"),
    ("fluid_cell_id", PI, "int32", 1, "fluid"),
    ("solid_position", PD, "float64", 2, "solid"),
    ("solid_reference_position", PD, "float64", 2, "solid"),
    ("solid_velocity", PD, "float64", 2, "solid"),
    ("solid_boundary_type", PI, "int32", 1, "solid"),
    ("solid_material_type", PI, "int32", 1, "solid"),
    ("solid_max_strain", PD, "float64", 4, "solid"),
    ("solid_pressure", PF, "float32", 1, "solid"),
    ("solid_deformation", PD, "float64", 4, "solid"),
    ("solid_stress_1st_piola", PD, "float64", 4, "solid"),
    ("solid_correction", PD, "float64", 4, "solid"),
    ("solid_du_dt", PD, "float64", 2, "solid"),
    ("solid_normal", PF, "float32", 2, "solid"),
    ("solid_couple_dudt", PF, "float32", 2, "solid"),
    ("solid_cell_id", PI, "int32", 1, "solid"),
    ("virt_position", PF, "float32", 2, "virt"),
    ("virt_normal", PF, "float32", 2, "virt"),
    ("virt_velocity", PF, "float32", 2, "virt"),
    ("virt_pressure", PF, "float32", 1, "virt"),
    ("virt_density", PF, "float32", 1, "virt"),
    ("virt_phase", PI, "int32", 1, "virt"),
    ("virt_boundary_type", PI, "int32", 1, "virt"),
    ("virt_cell_id", PI, "int32", 1, "virt"),
]

# the fields parsed from the .dat files (host_data.cuh:24-115)
INPUT_FIELDS = {
    "fluid_position", "fluid_velocity", "fluid_density", "fluid_pressure", "fluid_phase",
    "solid_position", "solid_velocity", "solid_reference_position", "solid_material_type",
    "solid_boundary_type", "virt_position", "virt_boundary_type",
}


class Tuning(C.Structure):
    """sphnj_tuning: the sweep configuration the autotuner chose."""
    _fields_ = [("tiled", C.c_int32), ("tile_h", C.c_int32), ("lists", C.c_int32), ("candidates", C.c_int32),
                ("ms_per_step", C.c_double), ("shift_block", C.c_int32), ("pair_block", C.c_int32),
                ("size_classes", C.c_int32), ("class_split", C.c_int32), ("class_tile_h", C.c_int32 * 2),
                ("class_lists", C.c_int32 * 2)]

    def as_dict(self) -> dict:
        return {"tiled": bool(self.tiled), "tile_h": self.tile_h, "lists": bool(self.lists),
                "candidates": self.candidates, "ms_per_step": self.ms_per_step,
                "shift_block": self.shift_block, "pair_block": self.pair_block,
                "size_classes": self.size_classes, "class_split": self.class_split,
                "class_tile_h": list(self.class_tile_h), "class_lists": [bool(x) for x in self.class_lists]}


class Diag(C.Structure):
    """sphnj_diag: global diagnostics reduced on the device in FP64."""
    _fields_ = [("step", C.c_int32), ("n_liquid", C.c_int32), ("front", C.c_double),
                ("fluid_momentum", C.c_double * 2), ("fluid_kinetic", C.c_double), ("fluid_mass", C.c_double),
                ("tip_disp", C.c_double * 2), ("solid_kinetic", C.c_double), ("solid_strain", C.c_double),
                ("total_force", C.c_double * 2), ("von_mises", C.c_double * 2), ("mean_pressure", C.c_double)]

    def as_dict(self) -> dict:
        out = {}
        for name, _ in self._fields_:
            v = getattr(self, name)
            out[name] = list(v) if hasattr(v, "__len__") else v
        return out


class HostState(C.Structure):
    _fields_ = [(name, ptr) for name, ptr, _, _, _ in STATE_FIELDS]


def count_of(p: Params, kind: str) -> int:
    return {"fluid": p.fluid_number_total, "solid": p.solid_number, "virt": p.virt_number}[kind]


def state_struct(arrays: dict) -> HostState:
    """HostState pointing into the given numpy arrays (missing -> NULL).
    The caller must keep the arrays alive while the struct is used."""
    import numpy as np

    s = HostState()
    for name, ptr, dtype, width, kind in STATE_FIELDS:
        a = arrays.get(name)
        if a is None:
            continue
        if not (isinstance(a, np.ndarray) and a.dtype == np.dtype(dtype) and a.flags.c_contiguous):
            raise TypeError(f"{name}: need a C-contiguous {dtype} array")
        setattr(s, name, a.ctypes.data_as(ptr))
    return s


class HostBlock:
    """One sphnj_host_alloc allocation (pinned, device-mapped host memory),
    freed when the last array viewing it is gone."""

    def __init__(self, lib, nbytes: int):
        self._lib = lib
        self.ptr = C.c_void_p()
        rc = lib.sphnj_host_alloc(max(int(nbytes), 1), C.byref(self.ptr))
        if rc:
            raise RuntimeError(f"sphnj_host_alloc({nbytes}) failed: {ERROR_NAMES.get(rc, rc)}")
        self.nbytes = max(int(nbytes), 1)

    def array(self, offset: int, shape, dtype):
        import numpy as np

        n = int(np.prod(shape)) * np.dtype(dtype).itemsize
        assert 0 <= offset and offset + n <= self.nbytes
        buf = (C.c_char * max(n, 1)).from_address(self.ptr.value + offset)
        buf.owner = self  # the ctypes buffer keeps the block alive
        return np.frombuffer(buf, dtype=dtype, count=int(np.prod(shape))).reshape(shape)

    def __del__(self):
        if getattr(self, "ptr", None) and self.ptr.value:
            self._lib.sphnj_host_free(self.ptr)
            self.ptr = C.c_void_p()


def alloc_state(p: Params, fields=None, lib=None) -> dict:
    """Zeroed host arrays of a state (all fields, or those named).  With the
    library given they share one sphnj_host_alloc block (pinned and
    device-mapped, each array 256-byte aligned), which the transfers move
    without copy-engine copies; otherwise they are ordinary numpy arrays."""
    import numpy as np

    spec = []
    for name, _, dtype, width, kind in STATE_FIELDS:
        if fields is not None and name not in fields:
            continue
        n = count_of(p, kind)
        spec.append((name, (n,) if width == 1 else (n, width), dtype))
    if lib is None:
        return {name: np.zeros(shape, dtype=dtype) for name, shape, dtype in spec}
    offs, total = [], 0
    for _, shape, dtype in spec:
        offs.append(total)
        total += (int(np.prod(shape)) * np.dtype(dtype).itemsize + 255) // 256 * 256
    block = HostBlock(lib, total)
    return {name: block.array(o, shape, dtype) for (name, shape, dtype), o in zip(spec, offs)}


def set_cells_args(cells):
    """Arguments of *_debug_set_cells from [(count, list)] * 3 (None = empty);
    returns (args, keepalive)."""
    import numpy as np

    args, keep = [], []
    for item in cells:
        if item is None:
            args += [None, None]
            continue
        cnt, lst = (np.ascontiguousarray(a, dtype=np.int32) for a in item)
        keep += [cnt, lst]
        args += [cnt.ctypes.data_as(PI), lst.ctypes.data_as(PI) if lst.size else None]
    return args, keep


def declare(lib: C.CDLL, prefix: str) -> None:
    """Set argtypes/restype for the context API under the given prefix
    ('sphnj' for the GPU library, 'oracle' for the CPU oracle)."""
    vp = C.c_void_p
    g = lambda n: getattr(lib, f"{prefix}_{n}")
    if prefix == "sphnj":
        g("create").argtypes = [C.POINTER(Params), C.c_int, C.POINTER(vp)]
        g("set_stream").argtypes = [vp, vp]
        g("set_stream").restype = C.c_int
        g("last_error").argtypes = [vp]
        g("last_error").restype = C.c_char_p
        g("synchronize").argtypes = [vp]
        g("synchronize").restype = C.c_int
        g("batch_create").argtypes = [C.POINTER(vp), C.c_int, C.POINTER(vp)]
        g("batch_destroy").argtypes = [vp]
        g("batch_destroy").restype = None
        g("batch_set_stream").argtypes = [vp, vp]
        g("batch_set_tiling").argtypes = [vp, C.c_int, C.c_int]
        g("batch_set_graphs").argtypes = [vp, C.c_int]
        PIi_ = C.POINTER(C.c_int)
        g("set_block_sizes").argtypes = [vp, C.c_int, C.c_int]
        g("get_block_sizes").argtypes = [vp, PIi_, PIi_]
        g("batch_set_block_sizes").argtypes = [vp, C.c_int, C.c_int]
        g("batch_set_scene_tiling").argtypes = [vp, C.c_int, C.c_int, C.c_int]
        g("batch_get_scene_tiling").argtypes = [vp, C.c_int, PIi_, PIi_]
        for n in ("set_block_sizes", "get_block_sizes", "batch_set_block_sizes", "batch_set_scene_tiling",
                  "batch_get_scene_tiling"):
            g(n).restype = C.c_int
        g("set_launch_chaining").argtypes = [vp, C.c_int]
        g("set_launch_chaining").restype = C.c_int
        g("batch_set_launch_chaining").argtypes = [vp, C.c_int]
        g("batch_set_launch_chaining").restype = C.c_int
        g("batch_step").argtypes = [vp, C.c_int]
        g("batch_synchronize").argtypes = [vp]
        g("batch_profile_enable").argtypes = [vp, C.c_int]
        g("batch_profile_read").argtypes = [vp, C.POINTER(C.c_double), C.POINTER(C.c_int64), C.POINTER(C.c_int64)]
        g("batch_stat_launches").argtypes = [vp, C.POINTER(C.c_uint64)]
        for n in ("batch_create", "batch_set_stream", "batch_set_tiling", "batch_set_graphs", "batch_step",
                  "batch_synchronize", "batch_profile_enable", "batch_profile_read", "batch_stat_launches"):
            g(n).restype = C.c_int
        g("batch_last_error").argtypes = [vp]
        g("batch_last_error").restype = C.c_char_p
        g("host_alloc").argtypes = [C.c_uint64, C.POINTER(vp)]
        g("host_alloc").restype = C.c_int
        g("host_free").argtypes = [vp]
        g("host_free").restype = C.c_int
        g("checkpoint_size").argtypes = [vp, C.POINTER(C.c_uint64)]
        g("checkpoint_save").argtypes = [vp, vp, C.c_uint64]
        g("checkpoint_load").argtypes = [vp, vp, C.c_uint64]
        g("checkpoint_write").argtypes = [vp, C.c_char_p]
        g("checkpoint_read").argtypes = [vp, C.c_char_p]
        for n in ("checkpoint_size", "checkpoint_save", "checkpoint_load", "checkpoint_write", "checkpoint_read"):
            g(n).restype = C.c_int
        g("diagnostics").argtypes = [vp, C.POINTER(Diag)]
        g("diagnostics").restype = C.c_int
        g("probe").argtypes = [vp, C.c_int, PF, PF]
        g("probe").restype = C.c_int
        PIi = C.POINTER(C.c_int)
        for pre in ("", "batch_"):
            g(pre + "set_neighbour_lists").argtypes = [vp, C.c_int]
            g(pre + "get_sweeps").argtypes = [vp, PIi, PIi, PIi]
            g(pre + "autotune").argtypes = [vp, C.c_int, C.POINTER(Tuning)]
            for n in ("set_neighbour_lists", "get_sweeps", "autotune"):
                g(pre + n).restype = C.c_int
    else:
        g("create").argtypes = [C.POINTER(Params), C.c_int, C.c_int, C.POINTER(vp)]
        g("error").argtypes = [vp]
        g("error").restype = C.c_int
        g("max_threads").argtypes = []
        g("max_threads").restype = C.c_int
        g("set_threads").argtypes = [C.c_int]
        g("set_threads").restype = C.c_int
        g("params_from_ini").argtypes = [C.c_char_p, PI, C.POINTER(Params)]
        g("params_from_ini").restype = C.c_int
    g("create").restype = C.c_int
    g("upload").argtypes = [vp, C.POINTER(HostState)]
    g("upload").restype = C.c_int
    g("step").argtypes = [vp, C.c_int]
    g("step").restype = C.c_int
    g("download").argtypes = [vp, C.c_uint32, C.POINTER(HostState)]
    g("download").restype = C.c_int
    g("debug_cells").argtypes = [vp, C.c_int, PI, PI, PI, PI]
    g("debug_cells").restype = C.c_int
    g("debug_max_speed").argtypes = [vp, PF]
    g("debug_max_speed").restype = C.c_int
    g("get_step").argtypes = [vp, PI]
    g("get_step").restype = C.c_int
    g("debug_set_cells").argtypes = [vp, PI, PI, PI, PI, PI, PI]
    g("debug_set_cells").restype = C.c_int
    g("debug_set_step").argtypes = [vp, C.c_int]
    g("debug_set_step").restype = C.c_int
    g("destroy").argtypes = [vp]
    g("destroy").restype = None
