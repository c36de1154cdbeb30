"""GPU (libsphnj through the C ABI) against the oracle and the reference.

Tolerances are relative to each field's scale (max |reference value|),
measured after ONE step from an identical state (lockstep tests re-sync the
complete state and cell lists before every step) or after a free run.  They
are set by the arithmetic difference between the two sides: the GPU
neighbour sweeps use __expf / __fdividef (as the reference's -use_fast_math
build does) and fused multiply-adds, the oracle IEEE expf and division
without contraction; per pair that is a ~1e-6 relative difference, which
cancellation in the momentum sum (pressure terms of size p/(rho h) summing
to ~g) amplifies to ~1e-4 of the field scale.
Integer work - cell ids, sorted order, per-cell lists - must be bit-exact.
"""
from __future__ import annotations

import numpy as np
import pytest

import sphnj_gb300 as S
from sphnj_gb300 import abi, cases

import oracle
from helpers import (CELL_IDS, FLUID_ENUMS, FLUID_FIELDS, SOLID_ENUMS, SOLID_FIELDS, VIRT_ENUMS, VIRT_FIELDS,
                     assert_lists_equal, cells_of, field_errors, golden, golden_case, golden_cells, golden_state,
                     load, nonempty, transfer)

pytestmark = pytest.mark.gpu

# one-step tolerances (relative to the field scale)
TOL_STEP = {
    "fluid_position": 2e-7, "fluid_velocity": 2e-4, "fluid_density": 2e-6, "fluid_pressure": 2e-4,
    "fluid_du_dx": 5e-4, "fluid_gradient": 5e-4, "fluid_du_dt": 5e-4, "fluid_color": 5e-5,
    "fluid_drho_dt": 5e-4,
    "solid_position": 1e-9, "solid_velocity": 1e-4, "solid_pressure": 5e-4, "solid_deformation": 1e-6,
    "solid_stress_1st_piola": 5e-4, "solid_correction": 1e-6, "solid_du_dt": 5e-4, "solid_normal": 1e-4,
    "solid_couple_dudt": 5e-4, "solid_max_strain": 1e-6,
    "virt_normal": 1e-5, "virt_velocity": 5e-4, "virt_pressure": 5e-4, "virt_density": 1e-5,
}


def enum_mismatches(a, b, names):
    return {n: int(np.sum(a[n] != b[n])) for n in names}


def check_step(g, o, p, what, tol_scale=1.0, enum_slack=0.002):
    sg, so = g.download(), o.download()
    for n in nonempty(p, CELL_IDS):
        assert np.array_equal(sg[n], so[n]), f"{what}: {n} differ at {np.sum(sg[n] != so[n])} particles"
    assert_lists_equal(g, o, p, what)
    names = nonempty(p, FLUID_FIELDS + SOLID_FIELDS + VIRT_FIELDS)
    errs = field_errors(sg, so, names, p)
    bad = {k: v for k, v in errs.items() if v > TOL_STEP[k] * tol_scale}
    assert not bad, f"{what}: field errors above tolerance {bad}"
    enums = nonempty(p, FLUID_ENUMS + SOLID_ENUMS + VIRT_ENUMS)
    mm = enum_mismatches(sg, so, enums)
    for n, m in mm.items():
        kind = n.split("_")[0]
        N = {"fluid": p.fluid_number_total, "solid": p.solid_number, "virt": p.virt_number}[kind]
        assert m <= max(2, enum_slack * N), f"{what}: {n} differs for {m} of {N} particles"
    return errs


LOCKSTEP_CASES = {
    "water": lambda: cases.dam_break_water(dx=0.02),
    "gas": lambda: cases.dam_break_gas(dx=0.05),
    "beam": lambda: cases.beam(dx=0.002, cfl=0.25),
    "gate": lambda: cases.gate(dx=0.002, gas=False, layers=3, substeps=4),
    # gas-liquid-solid: air at 1000:1 around the gate
    "gate_air": lambda: cases.gate(dx=0.002, gas=True, layers=3, substeps=4),
    "auxetic": lambda: cases.auxetic_block(dx=0.002, n=20),
}


@pytest.mark.parametrize("name", list(LOCKSTEP_CASES))
def test_lockstep_against_oracle(name):
    """Every step from an identical state: bit-exact cell ids / sort / lists,
    fields within TOL_STEP.  60 steps cover the sorts at steps 1 and 51 and
    the incremental rebuilds between them."""
    p, arr = load(LOCKSTEP_CASES[name]())
    o = oracle.OracleSim(p)
    o.upload(arr)
    with S.Simulation(p) as g:
        g.upload(o.download())  # includes the oracle's wall normals
        worst = {}
        for step in range(1, 61):
            if step > 1:
                transfer(o, g, p)
            o.step(1)
            g.step(1)
            g.synchronize()
            assert g.step_index == o.step_index == step
            errs = check_step(g, o, p, f"{name} step {step}")
            for k, v in errs.items():
                worst[k] = max(worst.get(k, 0.0), v)
            if p.fluid_number_total:
                assert abs(g.max_speed() - o.max_speed()) <= 1e-4 * max(o.max_speed(), 1e-12)
        print(name, {k: f"{v:.2e}" for k, v in sorted(worst.items())})


def test_wall_normals_match_oracle():
    p, arr = load(cases.dam_break_water(dx=0.02))
    o = oracle.OracleSim(p)
    o.upload(arr)
    with S.Simulation(p) as g:
        g.upload(arr)  # normals computed on the device (virt.cu:8-48)
        a, b = g.download(abi.F_VIRT), o.download(abi.F_VIRT)
        assert np.max(np.abs(a["virt_normal"] - b["virt_normal"])) < 1e-5


@pytest.mark.parametrize("name,steps,tol", [("water", 200, 2e-3), ("gate", 100, 2e-3), ("gate_air", 100, 2e-3),
                                           ("beam", 200, 1e-3)])
def test_free_run_against_oracle(name, steps, tol):
    """Independent runs from the same .dat input; differences grow with the
    step count, so the bound is looser than one step's."""
    p, arr = load(LOCKSTEP_CASES[name]())
    o = oracle.OracleSim(p)
    o.upload(arr)
    with S.Simulation(p) as g:
        g.upload(arr)
        o.step(steps)
        g.step(steps)
        g.synchronize()
        sg, so = g.download(), o.download()
    names = nonempty(p, ["fluid_position", "fluid_velocity", "fluid_density", "fluid_pressure",
                         "solid_position", "solid_velocity", "solid_deformation"])
    errs = field_errors(sg, so, names, p)
    bad = {k: v for k, v in errs.items() if v > tol}
    assert not bad, f"{name} after {steps} steps: {bad}"


@pytest.mark.parametrize("name,tile_h", [("water", 8), ("gas", 1), ("gas", 3), ("gate", 16), ("auxetic", 8)])
def test_tiled_sweeps_equal_per_particle_sweeps(name, tile_h):
    """The tiled neighbour sweeps sum the same terms in the same order as the
    one-thread-per-particle sweeps: the whole state is bit-identical after 60
    steps (two sorts and the rebuilds between them)."""
    p, arr = load(LOCKSTEP_CASES[name]())
    with S.Simulation(p) as a, S.Simulation(p) as b:
        a.set_tiling(False)
        b.set_tiling(True, tile_h)
        a.upload(arr)
        b.upload(arr)
        a.step(60)
        b.step(60)
        sa, sb = a.download(), b.download()
    for k in sa:
        assert np.array_equal(sa[k], sb[k], equal_nan=True), k


@pytest.mark.parametrize("name", ["gas", "gate"])
def test_graph_replay_equals_direct_launches(name):
    """Steps replayed from captured CUDA graphs give the same state, bit for
    bit, as launching every kernel directly (60 steps: sort and rebuild
    steps, both list buffers, the first virtual sort)."""
    p, arr = load(LOCKSTEP_CASES[name]())
    with S.Simulation(p) as a, S.Simulation(p) as b:
        a.set_graphs(False)
        b.set_graphs(True)
        a.upload(arr)
        b.upload(arr)
        for chunk in (1, 2, 7, 50):
            a.step(chunk)
            b.step(chunk)
        sa, sb = a.download(), b.download()
        assert a.launches() == b.launches()
    for k in sa:
        assert np.array_equal(sa[k], sb[k], equal_nan=True), k


def test_unlisted_particles_are_still_computed():
    """A particle that jumps two cells between sorts drops out of every cell
    list (pair.cu:66-154) but is still stepped (findFluidPair runs over all
    particle indices): the tiled sweeps leave it to the fallback kernels."""
    case = cases.dam_break_water(dx=0.05)
    p, arr = load(case)
    with S.Simulation(p) as a, S.Simulation(p) as b:
        a.set_tiling(False)
        for s in (a, b):
            s.upload(arr)
            s.step(3)
            st = s.download()
            st["fluid_position"][7] += np.float32(2.5 * p.interval[0])  # two cells to the right
            s.upload_fields(abi.F_FLUID_KINEMATICS, {"fluid_position": st["fluid_position"]})
            s.step(2)
        _, count, lst = b.cells(0)
        assert 7 not in set(lst.tolist())
        sa, sb = a.download(), b.download()
    for k in sa:
        assert np.array_equal(sa[k], sb[k], equal_nan=True), k


def test_sorted_order_and_partition():
    """After a sort step every particle is listed exactly once, in its own
    cell, in increasing index order, and cell ids are non-decreasing."""
    p, arr = load(cases.dam_break_gas(dx=0.05))
    with S.Simulation(p) as g:
        g.upload(arr)
        g.step(1)
        st = g.download(abi.F_CELL_IDS | abi.F_FLUID_KINEMATICS)
        cid = st["fluid_cell_id"]
        assert np.all(np.diff(cid) >= 0)
        start, count, lst = g.cells(0)
        assert np.array_equal(np.sort(lst), np.arange(p.fluid_number_total))
        for c in np.nonzero(count)[0][:200]:
            seg = lst[start[c]:start[c] + count[c]]
            assert np.all(cid[seg] == c) and np.all(np.diff(seg) > 0)


# ---- against the reference's own CUDA build ---------------------------------

GOLDEN_NAMES = ["water", "gas", "beam", "gate", "gate_air", "auxetic"]


@pytest.mark.parametrize("name", GOLDEN_NAMES)
def test_first_step_against_reference(name):
    """From the .dat input: step 1 (a sort step) reproduces the reference's
    cell ids, sorted order and lists bit-exactly, its wall normals, and its
    fields within the one-step tolerance."""
    g_ = golden(name)
    if g_ is None:
        pytest.skip("fixture not generated")
    case, gz = golden_case(name)
    p, arr = load(case)
    with S.Simulation(p) as g:
        g.upload(arr)
        if p.virt_number:
            ref_n = np.asarray(gz["s0/virt_normal"]).reshape(-1, 2)
            assert np.max(np.abs(g.download(abi.F_VIRT)["virt_normal"] - ref_n)) < 1e-5
        g.step(1)
        g.synchronize()
        _compare_to_golden(g, gz, 1, p, f"{name} step 1")


@pytest.mark.parametrize("name", GOLDEN_NAMES)
def test_incremental_step_against_reference(name):
    """From the reference's state and lists after step 51 (a sort step), the
    incremental rebuild of step 52 gives the reference's lists bit-exactly."""
    g_ = golden(name)
    if g_ is None:
        pytest.skip("fixture not generated")
    case, gz = golden_case(name)
    p, _ = load(case)
    with S.Simulation(p) as g:
        g.upload(golden_state(gz, 51, p))
        g.set_cells(*golden_cells(gz, 51, p))
        g.set_step(51)
        g.step(1)
        g.synchronize()
        _compare_to_golden(g, gz, 52, p, f"{name} step 52")


def _compare_to_golden(g, gz, step, p, what, tol_scale=4.0):
    sg = g.download()
    ref = golden_state(gz, step, p)
    for n in nonempty(p, CELL_IDS):
        assert np.array_equal(sg[n], ref[n]), f"{what}: {n} differ at {np.sum(sg[n] != ref[n])}"
    for k, (cnt, lst) in enumerate(golden_cells(gz, step, p)):
        _, count, got = g.cells(k)
        assert np.array_equal(count, cnt) and np.array_equal(got, lst), f"{what}: lists of kind {k} differ"
    names = nonempty(p, FLUID_FIELDS + SOLID_FIELDS + VIRT_FIELDS)
    errs = field_errors(sg, ref, names, p)
    bad = {k: v for k, v in errs.items() if v > TOL_STEP[k] * tol_scale}
    assert not bad, f"{what}: {bad}"


# ---- error paths (host-visible status codes, no device fault) ----------------

def test_out_of_grid_is_reported():
    """A solid particle outside the cell grid: the reference would index its
    cell array out of bounds; here the cell id is clamped and the status
    SPHNJ_ERR_OUT_OF_GRID is returned."""
    case = cases.beam(dx=0.004)
    case.solid_position[5] = [10.0, 10.0]
    case.solid_reference_position[5] = [10.0, 10.0]
    p, arr = load(case)
    with S.Simulation(p) as g:
        g.upload(arr)
        g.step(1)
        with pytest.raises(S.SphnjError) as e:
            g.synchronize()
        assert e.value.code == abi.ERR_OUT_OF_GRID


def test_cell_overflow_is_reported():
    """More than 64 particles in one cell (the reference's fixed capacity)."""
    case = cases.dam_break_water(dx=0.05)
    case.fluid_position[:80] = case.fluid_position[0] + np.linspace(0, 1e-3, 80, dtype=np.float32)[:, None]
    p, arr = load(case)
    with S.Simulation(p) as g:
        g.upload(arr)
        g.step(1)
        with pytest.raises(S.SphnjError) as e:
            g.synchronize()
        assert e.value.code == abi.ERR_CELL_OVERFLOW


@pytest.mark.parametrize("form", [abi.FORM_PLAIN, abi.FORM_MIXED])
def test_nonfinite_fluid_state_is_reported(form):
    """A NaN velocity injected on the host into an uploaded state: the
    reference steps on silently; here the fluid update flags it and the next
    synchronising call returns SPHNJ_ERR_NONFINITE (no device fault)."""
    p, arr = load(cases.dam_break_water(dx=0.05))
    arr["fluid_velocity"][11] = [np.nan, 0.0]  # into the uploaded host state
    with S.Simulation(p, form) as g:
        g.upload(arr)
        g.step(1)
        with pytest.raises(S.SphnjError) as e:
            g.synchronize()
        assert e.value.code == abi.ERR_NONFINITE


@pytest.mark.parametrize("form", [abi.FORM_PLAIN, abi.FORM_MIXED])
def test_nonfinite_solid_state_is_reported(form):
    p, arr = load(cases.beam(dx=0.004))
    # the tip, in the uploaded host state (the clamp's particles move at the fixed speed)
    arr["solid_velocity"][-1] = [0.0, np.inf]
    with S.Simulation(p, form) as g:
        g.upload(arr)
        g.step(1)
        with pytest.raises(S.SphnjError) as e:
            g.synchronize()
        assert e.value.code == abi.ERR_NONFINITE


def test_scene_in_a_batch_is_stepped_only_by_the_batch():
    """sphnj_step on a scene that belongs to a batch is refused (its step
    would move away from the batch's other scenes)."""
    p, arr = load(cases.dam_break_water(dx=0.05))
    with S.Simulation(p) as a, S.Simulation(p) as b:
        a.upload(arr)
        b.upload(arr)
        with S.Batch([a, b]) as bt:
            with pytest.raises(S.SphnjError) as e:
                a.step(1)
            assert e.value.code == abi.ERR_ARG
            bt.step(2)
            bt.synchronize()
            assert a.step_index == b.step_index == 2


@pytest.mark.parametrize("form", [abi.FORM_PLAIN, abi.FORM_MIXED], ids=["plain", "mixed"])
@pytest.mark.parametrize("name", ["gas", "gate_air"])
def test_launch_chaining_changes_nothing(name, form):
    """Programmatic dependent launch between a step's kernels (each kernel
    waits on the device for its predecessor) gives the same state, bit for
    bit, as plain stream-ordered launches, replayed from graphs or not."""
    p, arr = load(LOCKSTEP_CASES[name]())
    with S.Simulation(p, form) as a, S.Simulation(p, form) as b, S.Simulation(p, form) as c:
        a.set_launch_chaining(False)
        b.set_launch_chaining(True)
        c.set_launch_chaining(True)
        c.set_graphs(False)
        for s in (a, b, c):
            s.upload(arr)
            s.step(60)
        sa, sb, sc = a.download(), b.download(), c.download()
    for k in sa:
        assert np.array_equal(sa[k], sb[k], equal_nan=True), k
        assert np.array_equal(sa[k], sc[k], equal_nan=True), k
