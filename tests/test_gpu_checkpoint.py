"""Checkpoint / restart, the neighbour-list switch and the autotuner.

A checkpoint is the context's complete device state, so a run restored from
it continues bit-identically; the list switch and the tile height change only
how the sweeps are launched, so every configuration - and therefore the
autotuner's choice and its trial runs - leaves the results unchanged.
"""
from __future__ import annotations

import numpy as np
import pytest

import sphnj_gb300 as S
from sphnj_gb300 import abi, cases

from helpers import load

pytestmark = pytest.mark.gpu

CASES = {
    "gas": lambda: cases.dam_break_gas(dx=0.05),
    "gate": lambda: cases.gate(dx=0.002, gas=False, layers=3, substeps=4),
}


def same(a, b):
    for k in a:
        assert np.array_equal(a[k], b[k], equal_nan=True), k


@pytest.mark.parametrize("form", [abi.FORM_PLAIN, abi.FORM_MIXED])
@pytest.mark.parametrize("name", list(CASES))
def test_restart_from_checkpoint_file_is_bit_identical(name, form, tmp_path):
    p, arr = load(CASES[name]())
    path = tmp_path / "run.ck"
    with S.Simulation(p, form) as a:
        a.upload(arr)
        a.step(45)  # the restart crosses the sort at step 51
        a.save(path)
        a.step(20)
        ref = a.download()
        ref_step = a.step_index
    with S.Simulation(p, form) as b:
        b.load(path)
        assert b.step_index == 45
        b.step(20)
        assert b.step_index == ref_step
        same(ref, b.download())


def test_in_memory_restore_rewinds_the_run():
    p, arr = load(CASES["gate"]())
    with S.Simulation(p) as a:
        a.upload(arr)
        a.step(3)
        snap = a.checkpoint()
        a.step(10)
        first = a.download()
        a.restore(snap)
        a.step(10)
        same(first, a.download())


def test_checkpoint_of_another_layout_is_refused():
    p1, arr1 = load(CASES["gas"]())
    p2, arr2 = load(CASES["gate"]())
    with S.Simulation(p1) as a, S.Simulation(p2) as b, S.Simulation(p1, abi.FORM_MIXED) as c:
        a.upload(arr1)
        snap = a.checkpoint()
        with pytest.raises(S.SphnjError) as e:
            b.restore(snap)
        assert e.value.code == abi.ERR_ARG
        with pytest.raises(S.SphnjError):
            c.restore(snap)  # other form
        with pytest.raises(S.SphnjError) as e:
            b.restore(snap[:100])
        assert e.value.code == abi.ERR_IO


@pytest.mark.parametrize("form", [abi.FORM_PLAIN, abi.FORM_MIXED])
@pytest.mark.parametrize("name", list(CASES))
def test_stencil_walk_equals_stored_lists(name, form):
    """The stored lists visit the stencil walk's terms in its order, in both
    forms - also for the particles next to a wall, whose lists hold virtual
    slots (a quarter of the small gas tank's particles); the gate's particles
    next to the solid keep the walk."""
    p, arr = load(CASES[name]())
    out = []
    for lists in (True, False):
        with S.Simulation(p, form) as g:
            g.set_neighbour_lists(lists)
            assert g.sweeps()["lists"] == lists
            g.upload(arr)
            g.step(60)
            out.append(g.download())
    same(out[0], out[1])


@pytest.mark.parametrize("form", [abi.FORM_PLAIN, abi.FORM_MIXED])
def test_autotune_leaves_the_run_unchanged(form):
    p, arr = load(CASES["gas"]())
    with S.Simulation(p, form) as a, S.Simulation(p, form) as b:
        a.upload(arr)
        b.upload(arr)
        a.step(5)
        b.step(5)
        t = a.autotune(steps=3)
        # tile heights and lists, then 3 shifting-pass and 2 pair-pass block sizes
        assert t["candidates"] == (14 if t["tiled"] else 9) and t["ms_per_step"] > 0
        assert a.sweeps() == {"tiled": t["tiled"], "tile_h": t["tile_h"], "lists": t["lists"]}
        assert a.block_sizes() == (t["shift_block"], t["pair_block"]) and t["size_classes"] == 1
        assert a.step_index == b.step_index == 5
        if form == abi.FORM_PLAIN:
            # the plain form's sums do not depend on the launch shape
            a.step(10)
            b.step(10)
            same(b.download(), a.download())
        else:
            # the mixed form's tiled and per-particle frames round differently:
            # the run continues from exactly the tuned-from state
            b.set_tiling(t["tiled"], t["tile_h"])
            b.set_neighbour_lists(t["lists"])
            b.set_block_sizes(t["shift_block"], t["pair_block"])
            a.step(10)
            b.step(10)
            same(b.download(), a.download())


def test_batch_autotune():
    loaded = [load(cases.sweep_scene(s)) for s in (3, 9, 130, 200)]
    sims = [S.Simulation(p) for p, _ in loaded]
    for sim, (_, arr) in zip(sims, loaded):
        sim.upload(arr)
    ref = []
    for (p, arr) in loaded:
        with S.Simulation(p) as g:
            g.upload(arr)
            g.step(12)
            ref.append(g.download())
    with S.Batch(sims) as b:
        b.step(2)
        t = b.autotune(steps=3)
        # the two dam breaks form two size classes (the beams have no fluid)
        assert t["size_classes"] == 2 and t["class_split"] == max(p.fluid_number_total for p, _ in loaded)
        assert t["candidates"] == (9 + 3 + 2 + 2 * 4 if t["tiled"] else 9)
        small, large = (0, 1) if loaded[0][0].fluid_number_total < loaded[1][0].fluid_number_total else (1, 0)
        assert b.scene_tiling(small) == (t["class_tile_h"][0], t["class_lists"][0])
        assert b.scene_tiling(large) == (t["class_tile_h"][1], t["class_lists"][1])
        b.step(10)
        b.synchronize()
    for sim, r in zip(sims, ref):
        same(r, sim.download())
        sim.close()
