"""The GPU path (libsphnj through the C ABI) against the reference's own CUDA
build directly - no oracle in between - on the golden fixtures that
tests/golden/make_fixtures.py made by running the reference:

  - the late incremental step 199 -> 200 of the water dam break, from the
    reference's own state and lists (cell lists bit-exact, fields within the
    one-step tolerance of test_gpu_parity.py);
  - free runs of every fixture, in both forms, against the reference's
    global diagnostics over the whole run it made (2,000 steps for the water
    dam break and the cantilever, 200 for the others): surge front,
    momentum, kinetic energy, mass, beam-tip displacement, solid kinetic and
    strain energy, every 10 steps (5 for the auxetic block).

The diagnostics are computed on the host in float64 from downloaded states
with the definitions the reference harness uses (sphnj_gb300.diagnostics).
Tolerances are relative to each column's largest magnitude over the run.
"""
from __future__ import annotations

import numpy as np
import pytest

import sphnj_gb300 as S
from sphnj_gb300 import abi
from sphnj_gb300.diagnostics import COLUMNS, diagnostics

from helpers import golden, golden_case, golden_cells, golden_state, load, record
from test_gpu_parity import _compare_to_golden

pytestmark = pytest.mark.gpu

FLUID_COLS = ["front", "mom_x", "mom_y", "ek", "rho_sum"]
SOLID_COLS = ["eks", "eps"]
# name -> (steps compared, columns)
RUNS = {
    "water": (2000, FLUID_COLS),
    "beam": (2000, ["tip_x", "tip_y"] + SOLID_COLS),
    "gas": (200, FLUID_COLS),
    "gate": (200, FLUID_COLS + SOLID_COLS),
    "gate_air": (200, FLUID_COLS + SOLID_COLS),
    "auxetic": (200, ["tip_x"] + SOLID_COLS),
}
# relative to the column's scale over the run; the plain form computes in the
# reference's precision, the mixed form rounds differently (FP32 solid loops,
# cell + offset positions)
# (measured: plain at most 2.5e-5 - the gate's strain energy - and 1.4e-5 for
# the water's momentum over 2,000 steps; mixed at most 1.8e-4 - the gate's
# solid kinetic energy - and 1.0e-4 for the water's momentum)
TOL = {abi.FORM_PLAIN: {"fluid": 2e-4, "solid": 2e-4}, abi.FORM_MIXED: {"fluid": 1e-3, "solid": 1e-3}}


def test_late_step_against_reference():
    """Step 199 -> 200 of the water dam break, an incremental rebuild long
    after the last sort (step 151), from the reference's state and lists."""
    if golden("water") is None:
        pytest.skip("fixture not generated")
    case, gz = golden_case("water")
    p, _ = load(case)
    with S.Simulation(p) as g:
        g.upload(golden_state(gz, 199, p))
        g.set_cells(*golden_cells(gz, 199, p))
        g.set_step(199)
        g.step(1)
        g.synchronize()
        _compare_to_golden(g, gz, 200, p, "water step 200")


@pytest.mark.parametrize("form", [abi.FORM_PLAIN, abi.FORM_MIXED], ids=["plain", "mixed"])
@pytest.mark.parametrize("name", list(RUNS))
def test_trajectory_against_reference(name, form):
    if golden(name) is None:
        pytest.skip("fixture not generated")
    steps, cols = RUNS[name]
    case, gz = golden_case(name)
    p, arr = load(case)
    diag = np.asarray(gz["diag"])
    diag = diag[diag[:, 0] <= steps]
    scale = np.maximum(np.max(np.abs(diag), axis=0), 1e-30)
    worst = {c: 0.0 for c in cols}
    with S.Simulation(p, form) as g:
        g.upload(arr)
        done = 0
        for row in diag:
            s = int(row[0])
            if s > done:
                g.step(s - done)
                done = s
            if s == 0:
                continue
            mine = diagnostics(p, g.download(abi.F_FLUID_KINEMATICS | abi.F_FLUID_THERMO | abi.F_SOLID_KINEMATICS
                                             | abi.F_SOLID_DERIVED), s)
            for c in cols:
                k = COLUMNS.index(c)
                worst[c] = max(worst[c], abs(mine[k] - row[k]) / scale[k])
    form_name = "plain" if form == abi.FORM_PLAIN else "mixed"
    record(f"trajectory_vs_reference_{name}_{form_name}",
           {"case": name, "form": form_name, "steps": steps, "every": int(diag[1, 0] - diag[0, 0]),
            "max_rel_error": worst})
    tol = TOL[form]
    bad = {c: v for c, v in worst.items() if v > (tol["solid"] if c in SOLID_COLS or c.startswith("tip") else
                                                  tol["fluid"])}
    assert not bad, f"{name} ({form_name}) against the reference over {steps} steps: {bad}"
    print(name, form_name, {c: f"{v:.1e}" for c, v in worst.items()})
