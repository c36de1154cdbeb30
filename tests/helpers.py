"""Shared test helpers: case loading, state transfer between implementations,
and field comparison with stated tolerances."""
from __future__ import annotations

import tempfile
from pathlib import Path

import numpy as np

import sphnj_gb300 as S
from sphnj_gb300 import abi, cases

GOLDEN = Path(__file__).resolve().parent / "golden"

FLUID_FIELDS = ["fluid_position", "fluid_velocity", "fluid_density", "fluid_pressure", "fluid_du_dx",
                "fluid_gradient", "fluid_du_dt", "fluid_color", "fluid_drho_dt"]
FLUID_ENUMS = ["fluid_phase", "fluid_boundary_type", "fluid_has_near_particle"]
SOLID_FIELDS = ["solid_position", "solid_velocity", "solid_pressure", "solid_deformation",
                "solid_stress_1st_piola", "solid_correction", "solid_du_dt", "solid_normal",
                "solid_couple_dudt", "solid_max_strain"]
SOLID_ENUMS = ["solid_boundary_type", "solid_material_type"]
VIRT_FIELDS = ["virt_normal", "virt_velocity", "virt_pressure", "virt_density"]
VIRT_ENUMS = ["virt_phase", "virt_boundary_type"]
CELL_IDS = ["fluid_cell_id", "solid_cell_id", "virt_cell_id"]


def load(case: cases.Case):
    """Writes the case in the reference format and reads it back through the
    library's host I/O (the drop-in path)."""
    with tempfile.TemporaryDirectory() as t:
        case.write(t)
        return S.load_case(t)


def counts_of(p):
    return {"fluid": p.fluid_number_total, "solid": p.solid_number, "virt": p.virt_number}


def nonempty(p, names):
    c = counts_of(p)
    return [n for n in names if c[n.split("_")[0]] > 0]


def cells_of(sim, p):
    """[(count, list)] * 3 for set_cells, plus the start arrays."""
    out = []
    for k in range(3):
        start, count, lst = sim.cells(k)
        out.append((count, lst))
    return out


def transfer(src, dst, p):
    """Copies the complete state, cell lists and step counter of src into dst."""
    st = src.download()
    dst.upload(st)
    dst.set_cells(*cells_of(src, p))
    dst.set_step(src.step_index)
    return st


def norm_err(a, b, floor=0.0):
    """max |a - b| / max(max |b|, floor): the error relative to the field
    scale.  The floor is the field's physical scale, for fields that can be
    pure rounding noise (a kernel-gradient sum inside a completely filled
    domain, the stress of an undeformed solid)."""
    a = np.asarray(a, np.float64)
    b = np.asarray(b, np.float64)
    if a.size == 0:
        return 0.0
    scale = max(float(np.max(np.abs(b))), floor, 1e-30)
    return float(np.max(np.abs(a - b))) / scale


def floors(p) -> dict:
    """Physical scales of the fields that can vanish: 1/h for the kernel-
    gradient sum (a free-surface particle has |sum dx W'| ~ colour/h), 1e-6 E
    for stresses (strain 1e-6), the matching acceleration 1e-6 E/(rho_s h)."""
    h = float(p.smoothing_length)
    E = float(p.youngs_modulus)
    rs = float(p.solid_reference_density)
    return {"fluid_gradient": 1.0 / h, "solid_stress_1st_piola": 1e-6 * E, "solid_du_dt": 1e-6 * E / (rs * h),
            "fluid_du_dx": 1e-3 * float(max(p.sound_speed[0], p.sound_speed[1])) / h}


def field_errors(a: dict, b: dict, names, p=None) -> dict:
    fl = floors(p) if p is not None else {}
    return {n: norm_err(a[n], b[n], fl.get(n, 0.0)) for n in names}


def assert_lists_equal(sim_a, sim_b, p, what=""):
    for k, kind in enumerate(("fluid", "solid", "virt")):
        sa, ca, la = sim_a.cells(k)
        sb, cb, lb = sim_b.cells(k)
        assert np.array_equal(ca, cb), f"{what}: {kind} per-cell counts differ in {np.sum(ca != cb)} cells"
        assert np.array_equal(la, lb), f"{what}: {kind} cell lists differ at {np.sum(la != lb)} entries"


def golden(name):
    path = GOLDEN / f"{name}.npz"
    if not path.exists():
        return None
    return np.load(path, allow_pickle=False)


def golden_state(g, step, p):
    """Host-state dict of a reference dump (fields reshaped to the ABI)."""
    st = {}
    for name, ptr, dtype, width, kind in abi.STATE_FIELDS:
        key = f"s{step}/{name}"
        if key in g.files:
            a = np.asarray(g[key]).astype(dtype)
            st[name] = a.reshape(-1, width) if width > 1 else a
    return st


def golden_cells(g, step, p):
    cnt = np.asarray(g[f"s{step}/cell_counts"]).reshape(-1, 3)
    return [(cnt[:, 0].copy(), np.asarray(g[f"s{step}/cell_list_fluid"])),
            (cnt[:, 1].copy(), np.asarray(g[f"s{step}/cell_list_solid"])),
            (cnt[:, 2].copy(), np.asarray(g[f"s{step}/cell_list_virt"]))]


def golden_case(name):
    """Regenerates the case a fixture was made from (tests/golden/make_fixtures.py)."""
    import json

    g = golden(name)
    gen, kw = json.loads(str(g["generator"]))
    case = cases.by_name(gen, **kw)
    assert case.ini_text() == str(g["ini"]), f"{name}: generator output changed since the fixture was made"
    return case, g


def record(name: str, payload: dict):
    """Writes payload as <name>.json into $SPHNJ_RECORD_DIR when that is set
    (the measured errors of the long comparisons, kept beside the numbers
    they support); does nothing otherwise."""
    import json
    import os

    out = os.environ.get("SPHNJ_RECORD_DIR")
    if not out:
        return
    Path(out).mkdir(parents=True, exist_ok=True)
    (Path(out) / f"{name}.json").write_text(json.dumps(payload, indent=1, sort_keys=True) + "\n")
