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


def _states(loaded, steps, batched, tiled=True, graphs=True, chaining=True):
    sims = [S.Simulation(p) for p, _ in loaded]
    for sim, (_, arr) in zip(sims, loaded):
        sim.set_tiling(tiled)
        sim.set_graphs(graphs)
        sim.set_launch_chaining(chaining)
        sim.upload(arr)
    if batched:
        with S.Batch(sims) as b:
            b.set_tiling(tiled)
            b.set_graphs(graphs)
            b.set_launch_chaining(chaining)
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


def test_batch_launch_chaining_changes_nothing():
    """The batch's kernels chained by programmatic dependent launch give the
    same states, bit for bit, as plain launches."""
    names = list(MIXED)
    loaded = [load(MIXED[n]()) for n in names]
    steps = (1, 2, 7, 50, 3)
    plain, _, _ = _states(loaded, steps, batched=True, chaining=False)
    chained, _, _ = _states(loaded, steps, batched=True, chaining=True)
    _assert_same(plain, chained, names)


def test_scenes_with_their_own_tile_heights_equal_scenes_alone():
    """A batch whose scenes sweep tiles of different heights (8, 12, 24 and
    32 cells, lists off for one) and non-default block sizes gives every
    scene the state it has stepped alone with the default shape."""
    names = list(MIXED)
    loaded = [load(MIXED[n]()) for n in names]
    steps = (1, 2, 7, 50, 3)
    alone, _, _ = _states(loaded, steps, batched=False)
    sims = [S.Simulation(p) for p, _ in loaded]
    for sim, (_, arr) in zip(sims, loaded):
        sim.upload(arr)
    shapes = [(8, True), (12, True), (24, False), (32, True), (16, True), (8, False), (24, True)]
    with S.Batch(sims) as b:
        for k, (h, lists) in enumerate(shapes[:len(sims)]):
            b.set_scene_tiling(k, h, lists)
        b.set_block_sizes(64, 256)
        for chunk in steps:
            b.step(chunk)
        b.synchronize()
        assert b.scene_tiling(2) == (24, False)
    got = [sim.download(abi.F_ALL | abi.F_CELL_IDS) for sim in sims]
    for sim in sims:
        sim.close()
    _assert_same(alone, got, names)


@pytest.mark.parametrize("shift_threads,pair_threads", [(64, 128), (256, 256), (128, 0)])
def test_block_sizes_change_nothing(shift_threads, pair_threads):
    p, arr = load(MIXED["gas"]())
    with S.Simulation(p) as a, S.Simulation(p) as b:
        b.set_block_sizes(shift_threads, pair_threads)
        for s in (a, b):
            s.upload(arr)
            s.step(60)
        sa, sb = a.download(), b.download()
    for k in sa:
        assert np.array_equal(sa[k], sb[k], equal_nan=True), k


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
        # a scene of a batch is stepped, restored and given a stream only
        # through the batch: on its own it would leave the others behind
        with pytest.raises(S.SphnjError):
            sims[0].step(1)
        with pytest.raises(S.SphnjError):
            sims[0].restore(sims[0].checkpoint())
        with pytest.raises(S.SphnjError):
            sims[0].set_stream(None)
        b.step(1)
        b.synchronize()
        assert sims[0].step_index == sims[1].step_index == 4
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
