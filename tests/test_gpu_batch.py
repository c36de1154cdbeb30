"""Batched stepping (sphnj_batch_*) against the same scenes stepped alone.

A batch runs every stage of a step as one launch over all its scenes; each
scene's kernels, sums and order are the ones it runs alone, so the result of
every scene must be bit-identical to stepping that scene by itself - with
scenes of different sizes, particle kinds, shifting passes and solid
sub-steps in one batch, across sort and rebuild steps.
"""
from __future__ import annotations

import numpy as np
import pytest

import sphnj_gb300 as S
from sphnj_gb300 import abi, cases

from helpers import load

pytestmark = pytest.mark.gpu

MIXED = {
    "water": lambda: cases.dam_break_water(dx=0.02),
    "gas": lambda: cases.dam_break_gas(dx=0.05),
    "beam": lambda: cases.beam(dx=0.002, cfl=0.25),
    "gate": lambda: cases.gate(dx=0.002, gas=False, layers=3, substeps=4),
    "auxetic": lambda: cases.auxetic_block(dx=0.002, n=20),
    "sweep_dam": lambda: cases.sweep_scene(5),
    "sweep_beam": lambda: cases.sweep_scene(200),
}


def _states(loaded, steps, batched, tiled=True, graphs=True):
    sims = [S.Simulation(p) for p, _ in loaded]
    for sim, (_, arr) in zip(sims, loaded):
        sim.set_tiling(tiled)
        sim.set_graphs(graphs)
        sim.upload(arr)
    if batched:
        with S.Batch(sims) as b:
            b.set_tiling(tiled)
            b.set_graphs(graphs)
            for chunk in steps:
                b.step(chunk)
            b.synchronize()
            launches = b.launches()
    else:
        launches = 0
        for sim in sims:
            for chunk in steps:
                sim.step(chunk)
            sim.synchronize()
            launches += sim.launches()
    out = [sim.download(abi.F_ALL | abi.F_CELL_IDS) for sim in sims]
    cells = [[sim.cells(k) for k in range(3)] for sim in sims]
    for sim in sims:
        sim.close()
    return out, cells, launches


def _assert_same(a, b, names):
    for name, sa, sb in zip(names, a, b):
        for k in sa:
            assert np.array_equal(sa[k], sb[k], equal_nan=True), f"{name}: {k}"


@pytest.mark.parametrize("graphs", [True, False])
def test_batch_equals_scenes_stepped_alone(graphs):
    names = list(MIXED)
    loaded = [load(MIXED[n]()) for n in names]
    steps = (1, 2, 7, 50, 3)  # crosses the sort at step 51
    alone, cells_a, launches_alone = _states(loaded, steps, batched=False, graphs=graphs)
    batch, cells_b, launches = _states(loaded, steps, batched=True, graphs=graphs)
    _assert_same(alone, batch, names)
    for name, ca, cb in zip(names, cells_a, cells_b):
        for k in range(3):
            for x, y in zip(ca[k], cb[k]):
                assert np.array_equal(x, y), f"{name}: cell lists of kind {k}"
    # one launch per stage for the whole batch
    assert 0 < launches < launches_alone / 3


def test_batch_untiled_equals_tiled():
    names = ["gas", "sweep_dam", "gate"]
    loaded = [load(MIXED[n]()) for n in names]
    steps = (1, 10)
    tiled, _, _ = _states(loaded, steps, batched=True, tiled=True)
    untiled, _, _ = _states(loaded, steps, batched=True, tiled=False)
    _assert_same(tiled, untiled, names)


def test_batch_of_one_scene_equals_alone():
    loaded = [load(MIXED["gate"]())]
    alone, _, _ = _states(loaded, (5,), batched=False)
    batch, _, _ = _states(loaded, (5,), batched=True)
    _assert_same(alone, batch, ["gate"])


def test_batch_rejects_scenes_out_of_step():
    loaded = [load(MIXED[n]()) for n in ("water", "beam")]
    sims = [S.Simulation(p) for p, _ in loaded]
    for sim, (_, arr) in zip(sims, loaded):
        sim.upload(arr)
    sims[0].step(1)
    sims[0].synchronize()
    with pytest.raises(S.SphnjError):
        S.Batch(sims)
    sims[1].step(1)
    sims[1].synchronize()
    with S.Batch(sims) as b:
        b.step(2)
        # one scene stepped on its own leaves the batch out of step
        sims[0].step(1)
        with pytest.raises(S.SphnjError):
            b.step(1)
        with pytest.raises(S.SphnjError):
            sims[0].set_stream(None)
    for sim in sims:
        sim.close()


def test_batch_reports_the_failing_scene():
    good = load(MIXED["water"]())
    p, arr = load(MIXED["gas"]())
    arr = {k: v.copy() for k, v in arr.items()}
    arr["fluid_position"][7] = (1e4, 1e4)  # outside the cell grid
    sims = [S.Simulation(good[0]), S.Simulation(p)]
    sims[0].upload(good[1])
    sims[1].upload(arr)
    with S.Batch(sims) as b:
        b.step(1)
        with pytest.raises(S.SphnjError) as e:
            b.synchronize()
    assert e.value.code == abi.ERR_OUT_OF_GRID
    assert "scene 1" in str(e.value)
    for sim in sims:
        sim.close()
