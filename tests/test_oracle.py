"""The CPU oracle: pinned against the reference's own CUDA build (golden
fixtures from tests/golden/make_fixtures.py), FP32 against FP64, structural
invariants of the cell lists, and the error paths (planted on the CPU)."""
from __future__ import annotations

import numpy as np
import pytest

import oracle
from sphnj_gb300 import abi, cases
from sphnj_gb300.diagnostics import diagnostics

from helpers import (CELL_IDS, FLUID_FIELDS, SOLID_FIELDS, VIRT_FIELDS, field_errors, golden, golden_case,
                     golden_cells, golden_state, load, nonempty)

GOLDEN_NAMES = ["water", "gas", "beam", "gate", "gate_air", "auxetic"]

# oracle (IEEE float, no contraction) vs the reference build (-use_fast_math),
# one step from an identical state; relative to each field's scale
TOL_REF = {
    "fluid_position": 5e-7, "fluid_velocity": 1e-3, "fluid_density": 5e-6, "fluid_pressure": 1e-3,
    "fluid_du_dx": 2e-3, "fluid_gradient": 2e-3, "fluid_du_dt": 2e-3, "fluid_color": 2e-4,
    "fluid_drho_dt": 2e-3,
    "solid_position": 1e-9, "solid_velocity": 5e-4, "solid_pressure": 2e-3, "solid_deformation": 5e-6,
    "solid_stress_1st_piola": 2e-3, "solid_correction": 5e-6, "solid_du_dt": 2e-3, "solid_normal": 5e-4,
    "solid_couple_dudt": 2e-3, "solid_max_strain": 5e-6,
    "virt_normal": 5e-5, "virt_velocity": 2e-3, "virt_pressure": 2e-3, "virt_density": 5e-5,
}


def compare_golden(o, gz, step, p, what):
    so = o.download()
    ref = golden_state(gz, step, p)
    for n in nonempty(p, CELL_IDS):
        assert np.array_equal(so[n], ref[n]), f"{what}: {n} differ at {np.sum(so[n] != ref[n])} particles"
    for k, (cnt, lst) in enumerate(golden_cells(gz, step, p)):
        _, count, got = o.cells(k)
        assert np.array_equal(count, cnt), f"{what}: per-cell counts of kind {k} differ"
        assert np.array_equal(got, lst), f"{what}: cell lists of kind {k} differ"
    errs = field_errors(so, ref, nonempty(p, FLUID_FIELDS + SOLID_FIELDS + VIRT_FIELDS), p)
    bad = {k: v for k, v in errs.items() if v > TOL_REF[k]}
    assert not bad, f"{what}: {bad}"
    return errs


def need(name):
    if golden(name) is None:
        pytest.skip(f"golden fixture {name}.npz not generated")


@pytest.mark.parametrize("name", GOLDEN_NAMES)
def test_wall_normals_and_first_step_match_reference(name):
    need(name)
    case, gz = golden_case(name)
    p, arr = load(case)
    o = oracle.OracleSim(p)
    o.upload(arr)
    if p.virt_number:
        ref_n = np.asarray(gz["s0/virt_normal"]).reshape(-1, 2)
        assert np.max(np.abs(o.download(abi.F_VIRT)["virt_normal"] - ref_n)) < 5e-5
    o.step(1)
    assert o.error == 0
    compare_golden(o, gz, 1, p, f"{name} step 1")


@pytest.mark.parametrize("name", GOLDEN_NAMES)
def test_incremental_step_matches_reference(name):
    need(name)
    case, gz = golden_case(name)
    p, _ = load(case)
    o = oracle.OracleSim(p)
    o.upload(golden_state(gz, 51, p))
    o.set_cells(*golden_cells(gz, 51, p))
    o.set_step(51)
    o.step(1)
    compare_golden(o, gz, 52, p, f"{name} step 52")


def test_late_step_matches_reference():
    """Step 199 -> 200 of the water dam break (an incremental step long after
    the last sort at 151)."""
    need("water")
    case, gz = golden_case("water")
    p, _ = load(case)
    o = oracle.OracleSim(p)
    o.upload(golden_state(gz, 199, p))
    o.set_cells(*golden_cells(gz, 199, p))
    o.set_step(199)
    o.step(1)
    compare_golden(o, gz, 200, p, "water step 200")


def test_max_speed_matches_reference():
    need("water")
    case, gz = golden_case("water")
    p, arr = load(case)
    o = oracle.OracleSim(p)
    o.upload(arr)
    ms = np.asarray(gz["maxspeed"])
    for step in range(1, 31):
        o.step(1)
        ref = ms[ms[:, 0] == step, 1][0]
        assert abs(o.max_speed() - ref) <= 1e-4 * max(ref, 1e-12), (step, o.max_speed(), ref)


@pytest.mark.parametrize("name,steps,cols,tol", [
    ("water", 200, ["front", "mom_x", "mom_y", "ek", "rho_sum"], 2e-3),
    ("beam", 2000, ["tip_x", "tip_y", "eks", "eps"], 2e-2),
    ("gate_air", 200, ["front", "mom_x", "mom_y", "ek", "rho_sum", "eks", "eps"], 2e-3),
])
def test_trajectory_matches_reference(name, steps, cols, tol):
    """Free-running oracle against the reference's own diagnostics."""
    need(name)
    case, gz = golden_case(name)
    p, arr = load(case)
    o = oracle.OracleSim(p)
    o.upload(arr)
    diag = np.asarray(gz["diag"])
    from sphnj_gb300.diagnostics import COLUMNS

    done = 0
    for row in diag:
        s = int(row[0])
        if s > steps:
            break
        if s > done:
            o.step(s - done)
            done = s
        if s == 0:
            continue
        mine = diagnostics(p, o.download(), s)
        for c in cols:
            k = COLUMNS.index(c)
            scale = max(np.max(np.abs(diag[:, k])), 1e-30)
            assert abs(mine[k] - row[k]) <= tol * scale, (name, s, c, mine[k], row[k])


def test_fp32_against_fp64():
    """The reference-precision restatement stays close to the FP64 one."""
    p, arr = load(cases.dam_break_water(dx=0.05))
    a = oracle.OracleSim(p, oracle.REFERENCE_PRECISION)
    b = oracle.OracleSim(p, oracle.FP64)
    a.upload(arr)
    b.upload(arr)
    a.step(100)
    b.step(100)
    sa, sb = a.download(), b.download()
    assert np.max(np.abs(sa["fluid_position"] - sb["fluid_position"])) < 1e-4
    assert field_errors(sa, sb, ["fluid_pressure"])["fluid_pressure"] < 5e-2


def test_cell_lists_partition_and_order():
    """Each listed particle sits in the list of its own cell; after a sort the
    lists are contiguous index ranges; in between, every particle that moved
    at most one cell is listed exactly once."""
    p, arr = load(cases.dam_break_gas(dx=0.05))
    o = oracle.OracleSim(p)
    o.upload(arr)
    for step in range(1, 8):
        o.step(1)
        st = o.download(abi.F_CELL_IDS)
        start, count, lst = o.cells(0)
        cid = st["fluid_cell_id"]
        owner = np.repeat(np.arange(p.cell_number_total), count)
        assert np.all(cid[lst] == owner)
        assert len(np.unique(lst)) == len(lst)
        if step == 1:
            assert np.array_equal(lst, np.arange(p.fluid_number_total))


def test_hydrostatic_tank_stays_at_rest():
    """Water filling the tank width at hydrostatic pressure: velocities stay
    far below sqrt(g H)."""
    case = cases.tank("still", 0.05, 1.0, 1.0, 1.0, 0.6, layers=3, iend=300)
    p, arr = load(case)
    o = oracle.OracleSim(p)
    o.upload(arr)
    o.step(300)
    v = o.download()["fluid_velocity"]
    assert np.max(np.abs(v)) < 0.05 * np.sqrt(9.81 * 0.6)


def test_mass_and_phase_conserved():
    p, arr = load(cases.dam_break_gas(dx=0.05))
    o = oracle.OracleSim(p)
    o.upload(arr)
    o.step(60)
    st = o.download()
    assert int(np.sum(st["fluid_phase"] == abi.LIQUID)) == p.fluid_number[0]
    assert np.all(np.isfinite(st["fluid_position"]))


def test_cell_overflow_planted_on_cpu():
    case = cases.dam_break_water(dx=0.05)
    case.fluid_position[:80] = case.fluid_position[0] + np.linspace(0, 1e-3, 80, dtype=np.float32)[:, None]
    p, arr = load(case)
    o = oracle.OracleSim(p)
    o.upload(arr)
    with pytest.raises(oracle.OracleError):
        o.step(1)
    assert o.error == abi.ERR_CELL_OVERFLOW


def test_out_of_grid_planted_on_cpu():
    case = cases.beam(dx=0.004)
    case.solid_position[5] = [10.0, 10.0]
    p, arr = load(case)
    o = oracle.OracleSim(p)
    o.upload(arr)
    with pytest.raises(oracle.OracleError):
        o.step(1)
    assert o.error == abi.ERR_OUT_OF_GRID
