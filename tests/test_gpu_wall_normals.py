"""Wall normals (getVirtNormal, virt.cu:8-48) computed at upload from per-cell
lists of the virtual particles: against the oracle's O(N_v^2) index-order sum
on a tank with eight wall layers, and the step after an upload that computed
them is the step after an upload that was given them."""
from __future__ import annotations

import numpy as np
import pytest

import sphnj_gb300 as S
from sphnj_gb300 import abi, cases

import oracle

pytestmark = pytest.mark.gpu


def _tank(layers: int):
    case = cases.tank("walls", 0.01, 4.0, 3.0, 1.0, 2.0, layers=layers, iend=100, jitter=0.01, seed=7)
    return case.params(), case.arrays()


@pytest.mark.parametrize("layers", [3, 8])
def test_wall_normals_match_oracle(layers):
    p, arr = _tank(layers)
    assert p.virt_number > 1400 * layers
    with S.Simulation(p) as g:
        g.upload(arr)
        got = g.download(abi.F_VIRT)["virt_normal"].reshape(-1, 2)
    o = oracle.OracleSim(p)
    o.upload(arr)
    want = o.download()["virt_normal"].reshape(-1, 2)
    # The GPU weight uses __expf (as the reference's fast-math build), the
    # oracle IEEE expf; inside a thick wall the sum nearly cancels and its
    # direction magnifies that difference (5e-5 measured at three layers).
    # Against the reference's own build's normals the tolerance is 1e-5
    # (test_gpu_parity.py, test_first_step_against_reference).
    assert np.max(np.abs(got - want)) < 1e-4
    # unit normals where the sum is not below EPS_FOR_SUM
    nz = np.linalg.norm(want, axis=1) > 0.5
    assert np.all(np.abs(np.linalg.norm(got[nz], axis=1) - 1.0) < 1e-5)


@pytest.mark.parametrize("form", [abi.FORM_PLAIN, abi.FORM_MIXED])
def test_step_after_computed_normals_equals_step_after_given_normals(form):
    p, arr = _tank(3)
    with S.Simulation(p, form) as g:
        g.upload(arr)
        normals = g.download(abi.F_VIRT)["virt_normal"]
        g.step(3)
        g.synchronize()
        a = g.download()
    with S.Simulation(p, form) as g:
        g.upload(dict(arr, virt_normal=np.ascontiguousarray(normals)))
        g.step(3)
        g.synchronize()
        b = g.download()
    for k in a:
        assert np.array_equal(np.asarray(a[k]), np.asarray(b[k]), equal_nan=True), k
