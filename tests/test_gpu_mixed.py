"""Mixed-precision form (SPHNJ_FORM_MIXED) against the FP64 oracle.

The mixed form computes every pair loop in FP32 with positions held as an
integer cell + FP32 offset (Kahan-integrated), and solids in displacement
form with FP64 only for the correction-matrix inverse and the F / PK1 step.
It is not bit-identical to anything: its error is stated against the FP64
oracle (the oracle's double-precision build), next to the plain form's
error on the same run.  The targets are those of the benchmark statement:
beam-tip displacement and dam-break front within 0.5% of the FP64 oracle.
"""
from __future__ import annotations

import numpy as np
import pytest

import oracle
import sphnj_gb300 as S
from sphnj_gb300 import abi, cases
from sphnj_gb300.diagnostics import COLUMNS, diagnostics

from helpers import load

pytestmark = pytest.mark.gpu

MIXED = abi.FORM_MIXED
PLAIN = abi.FORM_PLAIN

CASES = {
    "water": lambda: cases.dam_break_water(dx=0.02),
    "gas": lambda: cases.dam_break_gas(dx=0.05),
    "beam": lambda: cases.beam(dx=0.002, cfl=0.25),
    "gate": lambda: cases.gate(dx=0.002, gas=False, layers=3, substeps=4),
    "auxetic": lambda: cases.auxetic_block(dx=0.002, n=20),
}


def gpu_run(p, arr, form, chunks, every=None):
    """Steps a GPU scene; returns the final state and (with `every`) the
    diagnostics sampled every `every` steps."""
    rows = []
    with S.Simulation(p, form) as g:
        g.upload(arr)
        done = 0
        for n in chunks:
            g.step(n)
            done += n
            if every:
                g.synchronize()
                rows.append(diagnostics(p, g.download(), done))
        g.synchronize()
        return g.download(), rows


def oracle_run(p, arr, chunks, every=None):
    rows = []
    o = oracle.OracleSim(p, oracle.FP64, threads=0)
    try:
        o.upload(arr)
        done = 0
        for n in chunks:
            o.step(n)
            done += n
            if every:
                rows.append(diagnostics(p, o.download(), done))
        return o.download(), rows
    finally:
        o.close()


def rel_err(a, b):
    a = np.asarray(a, np.float64)
    b = np.asarray(b, np.float64)
    scale = max(np.abs(b).max(), 1e-30)
    return float(np.abs(a - b).max() / scale)


def test_mixed_upload_download_round_trip():
    for name in ("gate", "beam", "water"):
        p, arr = load(CASES[name]())
        with S.Simulation(p, MIXED) as g:
            g.upload(arr)
            out = g.download()
        if p.fluid_number_total:
            # the offset holds a position to ~eps * cell width everywhere: FP32
            # positions come back exactly except within a few cell widths of
            # the origin, where absolute FP32 is finer than that
            atol = 2.0 ** -22 * max(p.interval[0], p.interval[1])
            np.testing.assert_allclose(out["fluid_position"], arr["fluid_position"], rtol=0, atol=atol)
            far = np.abs(arr["fluid_position"]).min(axis=1) > 8 * max(p.interval[0], p.interval[1])
            assert np.array_equal(out["fluid_position"][far], arr["fluid_position"][far]), name
        if p.solid_number:
            np.testing.assert_allclose(out["solid_position"], arr["solid_position"], rtol=0, atol=1e-15)
            np.testing.assert_allclose(out["solid_velocity"], arr["solid_velocity"], rtol=1e-7, atol=1e-12)


@pytest.mark.parametrize("name", list(CASES))
def test_mixed_and_plain_close_to_fp64_oracle(name):
    """A short free run (crossing a sort step): the largest per-field error
    of each GPU form against the FP64 oracle, relative to the field scale."""
    p, arr = load(CASES[name]())
    chunks = (1, 59)
    ref, _ = oracle_run(p, arr, chunks)
    mixed, _ = gpu_run(p, arr, MIXED, chunks)
    plain, _ = gpu_run(p, arr, PLAIN, chunks)
    fields = [f for f in ("fluid_position", "fluid_velocity", "fluid_density", "solid_position",
                          "solid_velocity") if f in ref and ref[f].size and np.abs(ref[f]).max() > 0]
    report = {}
    for f in fields:
        if f.endswith("position"):
            # positions: error relative to the particle spacing
            dx = float(p.particle_diameter)
            em = float(np.abs(mixed[f] - ref[f]).max()) / dx
            ep = float(np.abs(plain[f] - ref[f]).max()) / dx
        else:
            em, ep = rel_err(mixed[f], ref[f]), rel_err(plain[f], ref[f])
        report[f] = (em, ep)
        # after 60 steps both forms are within 1% of a particle spacing of the
        # FP64 oracle's positions and within 0.1% of its velocity / density
        # scale (measured: the mixed form's fluid positions are ~100x closer
        # than the plain form's; its FP32 solids ~100x further than the
        # plain form's FP64 solids, still < 1e-6 of the scale)
        assert em < (1e-2 if f.endswith("position") else 1e-3), (name, f, em, ep)
        assert ep < (1e-2 if f.endswith("position") else 1e-3), (name, f, em, ep)
    print(name, {k: f"mixed {v[0]:.2e} plain {v[1]:.2e}" for k, v in report.items()})


def test_beam_tip_within_half_percent_of_fp64():
    """Cantilever (E 1.4 MPa, nu 0.4, dx 2 mm): tip displacement over the
    first quarter period (to the largest deflection), sampled every 250
    steps: the mixed form within 0.5% of the FP64 oracle's amplitude."""
    case = cases.beam(dx=0.002, cfl=0.25)
    p, arr = load(case)
    period = 2 * np.pi / case.notes["omega1"]
    steps = int(0.25 * period / p.dt)
    chunks = [250] * (steps // 250)
    _, ref = oracle_run(p, arr, chunks, every=True)
    _, mixed = gpu_run(p, arr, MIXED, chunks, every=True)
    _, plain = gpu_run(p, arr, PLAIN, chunks, every=True)
    ty = COLUMNS.index("tip_y")
    r = np.array(ref)[:, ty]
    amp = np.abs(r).max()
    em = np.abs(np.array(mixed)[:, ty] - r).max() / amp
    ep = np.abs(np.array(plain)[:, ty] - r).max() / amp
    print(f"beam tip: amplitude {amp:.4e} m, mixed error {em:.2e}, plain error {ep:.2e} (of amplitude)")
    assert em < 5e-3
    assert ep < 5e-3


@pytest.mark.parametrize("form", [PLAIN, MIXED])
def test_cantilever_period_matches_euler_bernoulli(form):
    """Analytical check: the cantilever (clamped over 0.06 m, E 1.4 MPa,
    nu 0.4, L 0.2 m, thickness 0.02 m) set off in its first bending mode
    oscillates with the Euler-Bernoulli first-mode period 2 pi / omega_1,
    omega_1 = 1.875^2 sqrt(E t^2 / (12 rho)) / L^2.  The tip displacement is
    sampled from the device diagnostics; its period is taken between its
    first two zero crossings.  A thick (L/t = 10) 2-D SPH beam is softer than
    slender-beam theory - shear deformation and the compliance of a clamp made
    of particles - so its period is longer: measured +8.8% in both forms,
    inside the 10% band."""
    case = cases.beam(dx=0.002, cfl=0.25)
    p, arr = load(case)
    period = 2 * np.pi / case.notes["omega1"]
    every = 100
    n = int(1.3 * period / p.dt / every)
    t, tip = [], []
    with S.Simulation(p, form) as g:
        g.upload(arr)
        for _ in range(n):
            g.step(every)
            dg = g.diagnostics()
            t.append(dg["step"] * p.dt)
            tip.append(dg["tip_disp"][1])
    t, tip = np.array(t), np.array(tip)
    cross = [t[k] - tip[k] * (t[k + 1] - t[k]) / (tip[k + 1] - tip[k])
             for k in range(len(tip) - 1) if tip[k] != 0 and np.sign(tip[k]) != np.sign(tip[k + 1])]
    assert len(cross) >= 2, cross
    measured = 2.0 * (cross[1] - cross[0])
    print(f"form {form}: period {measured:.5f} s, Euler-Bernoulli {period:.5f} s "
          f"({100 * (measured / period - 1):+.2f}%)")
    assert abs(measured / period - 1.0) < 0.10


def test_water_front_within_half_percent_of_fp64():
    """Water dam break at dx 0.02 (5,000 particles) for 2,000 steps: the
    surge front of the mixed form within 0.5% of the FP64 oracle's, sampled
    every 200 steps."""
    p, arr = load(cases.dam_break_water(dx=0.02))
    chunks = [200] * 10
    _, ref = oracle_run(p, arr, chunks, every=True)
    _, mixed = gpu_run(p, arr, MIXED, chunks, every=True)
    _, plain = gpu_run(p, arr, PLAIN, chunks, every=True)
    fr = COLUMNS.index("front")
    r = np.array(ref)[:, fr]
    em = np.abs(np.array(mixed)[:, fr] - r).max() / np.abs(r).max()
    ep = np.abs(np.array(plain)[:, fr] - r).max() / np.abs(r).max()
    print(f"water front: mixed error {em:.2e}, plain error {ep:.2e} (relative)")
    assert em < 5e-3
    assert ep < 5e-3


def test_mixed_batch_equals_scenes_alone():
    names = ["water", "beam", "gate", "auxetic"]
    loaded = [load(CASES[n]()) for n in names]
    alone = []
    for p, arr in loaded:
        st, _ = gpu_run(p, arr, MIXED, (1, 7, 50, 2))
        alone.append(st)
    sims = [S.Simulation(p, MIXED) for p, _ in loaded]
    for sim, (_, arr) in zip(sims, loaded):
        sim.upload(arr)
    with S.Batch(sims) as b:
        for n in (1, 7, 50, 2):
            b.step(n)
        b.synchronize()
    for name, sim, a in zip(names, sims, alone):
        got = sim.download()
        for k in a:
            assert np.array_equal(a[k], got[k], equal_nan=True), (name, k)
        sim.close()


def test_mixed_tiled_close_to_untiled():
    """The tiled sweep works in the tile's frame, the per-particle sweep in
    each particle's own cell frame: the same sums with different rounding."""
    p, arr = load(CASES["gas"]())
    out = {}
    for tiled in (True, False):
        with S.Simulation(p, MIXED) as g:
            g.set_tiling(tiled)
            g.upload(arr)
            g.step(5)
            out[tiled] = g.download()
    for f in ("fluid_position", "fluid_velocity", "fluid_density"):
        assert rel_err(out[True][f], out[False][f]) < 1e-5, f


def test_mixed_out_of_grid_is_reported():
    case = cases.beam(dx=0.004)
    case.solid_position[5] = [10.0, 10.0]
    case.solid_reference_position[5] = [10.0, 10.0]
    p, arr = load(case)
    with S.Simulation(p, MIXED) as g:
        with pytest.raises(S.SphnjError) as e:
            g.upload(arr)
            g.step(1)
            g.synchronize()
        assert e.value.code == abi.ERR_OUT_OF_GRID
