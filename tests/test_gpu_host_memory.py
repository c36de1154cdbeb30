"""Transfers through pinned, device-mapped host memory (sphnj_host_alloc).

Fluid positions, velocities, densities and pressures held in such memory are
moved by one kernel over the host link (with the mixed form's split and join
on the way); everything else, and any array that is not wholly inside one
allocation or not aligned for the kernel, takes the copy-engine path.  The
two paths must leave the same state and return the same bytes.
"""
from __future__ import annotations

import ctypes as C

import numpy as np
import pytest

import sphnj_gb300 as S
from sphnj_gb300 import abi, cases

from helpers import load

pytestmark = pytest.mark.gpu

IO = ("fluid_position", "fluid_velocity", "fluid_density", "fluid_pressure")
MASK = abi.F_FLUID_KINEMATICS | abi.F_FLUID_THERMO


def same(a, b, names=None):
    for k in names or a:
        assert np.array_equal(a[k], b[k], equal_nan=True), k


def case():
    return load(cases.dam_break_gas(dx=0.05))


@pytest.mark.parametrize("form", [abi.FORM_PLAIN, abi.FORM_MIXED])
def test_mapped_download_equals_copy_download(form):
    p, arr = case()
    with S.Simulation(p, form) as a:
        a.upload(arr)
        a.step(30)
        mapped = a.download(MASK, into=a.host_state(IO))
        plain = a.download(MASK, into=S.alloc_state(p, IO))
        same(plain, mapped)
        # the mapped download left the device state as the copy path does
        after_a = a.download()
    with S.Simulation(p, form) as b:
        b.upload(arr)
        b.step(30)
        b.download(MASK, into=S.alloc_state(p, IO))
        same(b.download(), after_a)


@pytest.mark.parametrize("form", [abi.FORM_PLAIN, abi.FORM_MIXED])
@pytest.mark.parametrize("fields", [IO, ("fluid_density",), ("fluid_position",), ("fluid_velocity",),
                                    ("fluid_velocity", "fluid_pressure")])
def test_mapped_upload_equals_copy_upload(form, fields):
    """Overwrite some fluid fields mid-run through either path, step on, and
    compare the whole state: same split, same compensation resets."""
    p, arr = case()
    rng = np.random.default_rng(3)
    outs = []
    for use_mapped in (False, True):
        with S.Simulation(p, form) as sim:
            sim.upload(arr)
            sim.step(12)
            cur = sim.download(MASK, into=S.alloc_state(p, IO))
            new = {k: cur[k].copy() for k in fields}
            if "fluid_position" in new:
                new["fluid_position"] += rng.uniform(-1e-4, 1e-4, new["fluid_position"].shape).astype(np.float32)
            if "fluid_velocity" in new:
                new["fluid_velocity"] *= np.float32(0.99)
            if "fluid_density" in new:
                new["fluid_density"] *= np.float32(1.0001)
            if "fluid_pressure" in new:
                new["fluid_pressure"] += np.float32(1.0)
            rng = np.random.default_rng(3)  # the same perturbation for both paths
            if use_mapped:
                host = sim.host_state(fields)
                for k in fields:
                    host[k][...] = new[k]
                new = host
            sim.upload_fields(MASK, new)
            sim.step(15)
            outs.append(sim.download())
    same(outs[0], outs[1])


def test_misaligned_arrays_take_the_copy_path():
    """A float2 array at a 4-byte offset inside a block is refused by the
    kernel path (its float2 accesses would be misaligned) and still moves
    correctly through the copy engines, both ways."""
    p, arr = case()
    nf = p.fluid_number_total
    block = abi.HostBlock(S.lib(), 8 * nf + 16)
    pos = block.array(4, (nf, 2), np.float32)  # 4-byte aligned only
    assert pos.ctypes.data % 8 == 4
    with S.Simulation(p, abi.FORM_MIXED) as a:
        a.upload(arr)
        a.step(5)
        ref = a.download(abi.F_FLUID_KINEMATICS, into=S.alloc_state(p, ("fluid_position",)))
        got = a.download(abi.F_FLUID_KINEMATICS, into={"fluid_position": pos})
        same(ref, got)
        pos[...] += np.float32(1e-4)
        a.upload_fields(abi.F_FLUID_KINEMATICS, {"fluid_position": pos})
        back = a.download(abi.F_FLUID_KINEMATICS, into=S.alloc_state(p, ("fluid_position",)))
        # one split and one join: within an FP32 rounding of the input
        np.testing.assert_allclose(back["fluid_position"], pos, rtol=0, atol=2e-6)



@pytest.mark.parametrize("form", [abi.FORM_PLAIN, abi.FORM_MIXED])
@pytest.mark.parametrize("mapped", [False, True])
def test_step_exchange_equals_separate_calls(form, mapped):
    """sphnj_step_exchange (upload, n steps, download in one call, its
    transfers overlapped with the steps) gives exactly what the three calls
    give, through a sort step, round-tripping the state through the host."""
    p, arr = case()
    runs = []
    for exchange in (False, True):
        with S.Simulation(p, form) as sim:
            sim.upload(arr)
            sim.step(3)
            hin = sim.host_state(IO) if mapped else S.alloc_state(p, IO)
            hout = sim.host_state(IO) if mapped else S.alloc_state(p, IO)
            sim.download(MASK, into=hin)
            seq = []
            for it in range(4):  # steps 4..63: the sort step 51 inside
                hin["fluid_velocity"] *= np.float32(0.999)
                hin["fluid_pressure"] += np.float32(0.5)
                if exchange:
                    sim.step_exchange(15, MASK, hin, MASK, hout)
                else:
                    sim.upload_fields(MASK, hin)
                    sim.step(15)
                    sim.download(MASK, into=hout)
                seq.append({k: v.copy() for k, v in hout.items()})
                hin, hout = hout, hin
            runs.append((seq, sim.download(), sim.step_index))
    (sa, fa, ia), (sb, fb, ib) = runs
    assert ia == ib == 63
    for a, b in zip(sa, sb):
        same(a, b)
    same(fa, fb)


@pytest.mark.parametrize("form", [abi.FORM_PLAIN, abi.FORM_MIXED])
def test_step_exchange_one_way(form):
    """Upload only, download only, and a velocity-only upload (the mixed
    form's compensation reset) through sphnj_step_exchange."""
    p, arr = case()
    runs = []
    for exchange in (False, True):
        with S.Simulation(p, form) as sim:
            sim.upload(arr)
            sim.step(2)
            v = sim.download(abi.F_FLUID_KINEMATICS, into=S.alloc_state(p, ("fluid_velocity",)))
            v["fluid_velocity"] *= np.float32(1.01)
            got = S.alloc_state(p, ("fluid_density", "fluid_pressure"))
            if exchange:
                sim.step_exchange(4, abi.F_FLUID_KINEMATICS, v, 0, None)
                sim.step_exchange(3, 0, None, abi.F_FLUID_THERMO, got)
            else:
                sim.upload_fields(abi.F_FLUID_KINEMATICS, v)
                sim.step(4)
                sim.step(3)
                sim.download(abi.F_FLUID_THERMO, into=got)
            runs.append((got, sim.download()))
    same(runs[0][0], runs[1][0])
    same(runs[0][1], runs[1][1])


@pytest.mark.parametrize("form", [abi.FORM_PLAIN, abi.FORM_MIXED])
def test_step_exchange_without_graphs_and_while_profiling(form):
    """The exchange's event waits and records also order direct launches
    (graphs off) and the timed stages of profiling."""
    p, arr = case()
    runs = []
    for mode in ("graphs", "direct", "profiled"):
        with S.Simulation(p, form) as sim:
            if mode == "direct":
                sim.set_graphs(False)
            if mode == "profiled":
                sim.profile_enable(True)
            sim.upload(arr)
            sim.step(2)
            h = sim.host_state(IO)
            sim.download(MASK, into=h)
            for _ in range(3):
                h["fluid_pressure"] *= np.float32(1.001)
                sim.step_exchange(20, MASK, h, MASK, h)
            runs.append(sim.download())
    same(runs[0], runs[1])
    same(runs[0], runs[2])


def test_step_exchange_refuses_a_batched_scene():
    loaded = [load(cases.sweep_scene(s)) for s in (3, 9)]
    sims = [S.Simulation(p, abi.FORM_MIXED) for p, _ in loaded]
    try:
        for sim, (_, arr) in zip(sims, loaded):
            sim.upload(arr)
        with S.Batch(sims):
            with pytest.raises(S.SphnjError):
                sims[0].step_exchange(1, 0, None, 0, None)
    finally:
        for sim in sims:
            sim.close()
