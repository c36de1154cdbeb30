"""The host driver (sphnj_run), device diagnostics and probes on the GPU.

The driver's files are checked against the library run directly; the
diagnostics (FP64 device reductions) against the same quantities recomputed
on the host from a download, with the reference's definitions
(output.cu:283-560); probes against a host Shepard sum over the cell lists.
"""
from __future__ import annotations

import subprocess
from pathlib import Path

import numpy as np
import pytest

import sphnj_gb300 as S
from sphnj_gb300 import _build, abi, cases

from helpers import load

pytestmark = pytest.mark.gpu


def read_vtk(path: Path):
    lines = Path(path).read_text().splitlines()
    assert lines[0] == "# vtk DataFile Version 2.0"
    assert lines[2] == "ASCII" and lines[3] == "DATASET POLYDATA"
    n = int(lines[4].split()[1])
    pts = np.array([[float(v) for v in l.split()] for l in lines[5:5 + n]])
    assert lines[5 + n] == f"POINT_DATA {n}"
    kind = lines[6 + n].split()[0]
    start = 7 + n if kind == "VECTORS" else 8 + n
    vals = np.array([[float(v) for v in l.split()] for l in lines[start:start + n]])
    assert len(lines) == start + n
    return pts, vals


def g6(x):
    return np.array([float(f"{float(v):.6g}") for v in np.ravel(x)]).reshape(np.shape(x))


def run_driver(case_dir, *args):
    S.build()
    r = subprocess.run([str(_build.DRIVER), str(case_dir), "--quiet", *args], capture_output=True, text=True,
                       timeout=600)
    assert r.returncode == 0, r.stderr
    return r


def test_driver_water_outputs_match_the_library(tmp_path):
    case = cases.dam_break_water(dx=0.05, iend=200)
    case.ini["result_interval"] = "100"
    cdir = case.write(tmp_path / "water")
    run_driver(cdir, "--global", "frontier,total_energy,total_force,tip_disp", "--probe", "0.5,0.5",
               "--probe", "3.5,0.2")
    out = cdir / "out"
    for fs in (0, 1, 2):  # i = 1, 101 and the final output at i = iend + 1
        for f in ("fluid_velocity", "fluid_density", "fluid_pressure"):
            assert (out / "fluid" / f"{f}-{fs}.vtk").exists()
        assert (out / "virtual" / f"virt_normal-{fs}.vtk").exists()
    assert not (out / "fluid" / "fluid_pressure-3.vtk").exists()
    p, arr = load(case)
    with S.Simulation(p) as g:
        g.upload(arr)
        g.step(100)
        st = g.download()
    pts, vals = read_vtk(out / "fluid" / "fluid_pressure-1.vtk")
    np.testing.assert_array_equal(pts[:, :2], g6(st["fluid_position"]))
    np.testing.assert_array_equal(vals[:, 0], g6(st["fluid_pressure"]))
    _, dens = read_vtk(out / "fluid" / "fluid_density-1.vtk")
    liq = st["fluid_phase"] == abi.LIQUID
    np.testing.assert_array_equal(dens[liq, 0], st["fluid_boundary_type"][liq])
    gl = out / "global"
    for name in ("frontier", "total_energy", "total_force", "tip_disp", "probe-0", "probe-1"):
        assert len((gl / f"{name}.dat").read_text().splitlines()) == 200, name
    probe = np.loadtxt(gl / "probe-0.dat")
    assert probe.shape == (200, 6) and np.all(probe[:, 0] == np.float32(0.5))


def test_driver_restart_reproduces_the_run(tmp_path):
    case = cases.gate(dx=0.004, gas=False, layers=3, substeps=4, iend=60)
    case.ini["result_interval"] = "60"
    a = case.write(tmp_path / "a")
    b = case.write(tmp_path / "b")
    for form in ("plain", "mixed"):
        run_driver(a, "--form", form, "--checkpoint-every", "30", "--global-every", "0")
        ck = a / "out" / "checkpoint-30.bin"
        assert ck.exists()
        run_driver(b, "--form", form, "--restart", str(ck), "--global-every", "0")
        for sub, f in (("fluid", "fluid_velocity"), ("solid", "solid_velocity"), ("solid", "solid_stress"),
                       ("virtual", "virt_pressure")):
            ta = (a / "out" / sub / f"{f}-1.vtk").read_text()
            tb = (b / "out" / sub / f"{f}-1.vtk").read_text()
            assert ta == tb, (form, f)
        _, stress = read_vtk(a / "out" / "solid" / "solid_stress-1.vtk")
        assert np.all(stress == 0.0)  # LINEAR_ELASTIC rows are written as 0.0 0.0 0.0


def host_diag(p, st):
    d = float(np.float32(p.particle_diameter))
    dv = float(np.float32(p.particle_diameter)) ** 2
    out = {}
    if p.fluid_number_total:
        x = st["fluid_position"].astype(np.float64)
        v = st["fluid_velocity"].astype(np.float64)
        ph = st["fluid_phase"]
        m = np.where(ph == abi.GAS, float(np.float32(p.reference_density[1])),
                     float(np.float32(p.reference_density[0]))) * dv
        liq = ph == abi.LIQUID
        out["front"] = x[liq, 0].max() + 0.5 * d
        out["fluid_momentum"] = [np.sum(m * v[:, 0]), np.sum(m * v[:, 1])]
        out["fluid_kinetic"] = np.sum(0.5 * m * np.sum(v * v, axis=1))
        out["fluid_mass"] = np.sum(st["fluid_density"].astype(np.float64)) * dv
    if p.solid_number:
        X, x, v = st["solid_reference_position"], st["solid_position"], st["solid_velocity"]
        F = st["solid_deformation"].reshape(-1, 4)
        P = st["solid_stress_1st_piola"].reshape(-1, 4)
        mat = st["solid_material_type"]
        cand = np.nonzero(X[:, 0] >= X[:, 0].max() - 1e-12)[0]
        best = cand[np.argmin(np.abs(X[cand, 1] - X[:, 1].mean()))]
        out["tip_disp"] = list(x[best] - X[best])
        lam, mu = float(np.float32(p.lambda_)), float(np.float32(p.nu))
        e00 = 0.5 * (F[:, 0] ** 2 + F[:, 1] ** 2 - 1)
        e11 = 0.5 * (F[:, 2] ** 2 + F[:, 3] ** 2 - 1)
        e01 = 0.5 * (F[:, 0] * F[:, 2] + F[:, 1] * F[:, 3])
        out["solid_strain"] = np.sum((0.5 * lam * (e00 + e11) ** 2 + mu * (e00 ** 2 + e11 ** 2 + 2 * e01 ** 2)) * dv)
        rho_s = float(np.float32(p.solid_reference_density))
        keep = X[:, 0] >= 0.0
        out["solid_kinetic"] = np.sum(0.5 * rho_s * dv * np.sum(v[keep] ** 2, axis=1))
        rho = np.where(mat == abi.LINEAR_ELASTIC, rho_s, float(np.float32(p.auxetic_density)))
        cf = st["solid_couple_dudt"].astype(np.float64)
        out["total_force"] = [np.sum(cf[:, 0] * dv * rho), np.sum(cf[:, 1] * dv * rho)]
        det = F[:, 0] * F[:, 3] - F[:, 1] * F[:, 2]
        i00, i10, i01, i11 = F[:, 3] / det, -F[:, 1] / det, -F[:, 2] / det, F[:, 0] / det
        s00 = i00 * P[:, 0] + i01 * P[:, 1]
        s11 = i10 * P[:, 2] + i11 * P[:, 3]
        s01 = i00 * P[:, 2] + i01 * P[:, 3]
        vm = np.sqrt(0.5 * (s00 - s11) ** 2 + 3 * s01 ** 2)
        out["von_mises"] = [vm[mat == abi.LINEAR_ELASTIC].max(initial=0.0), vm[mat == abi.AUXETIC].max(initial=0.0)]
        out["mean_pressure"] = np.mean(st["solid_pressure"].astype(np.float64))
    return out


@pytest.mark.parametrize("form", [abi.FORM_PLAIN, abi.FORM_MIXED])
@pytest.mark.parametrize("name", ["gas", "gate", "beam", "auxetic"])
def test_device_diagnostics_match_host(name, form):
    case = {"gas": lambda: cases.dam_break_gas(dx=0.05),
            "gate": lambda: cases.gate(dx=0.002, gas=False, layers=3, substeps=4),
            "beam": lambda: cases.beam(dx=0.002, cfl=0.25),
            "auxetic": lambda: cases.auxetic_block(dx=0.002, n=20)}[name]()
    p, arr = load(case)
    with S.Simulation(p, form) as g:
        g.upload(arr)
        g.step(30)
        dev = g.diagnostics()
        st = g.download()
    assert dev["step"] == 30
    ref = host_diag(p, st)
    # the mixed form's host copy rounds positions to FP32 / joins FP64 from
    # float parts: its position-based sums agree to that rounding
    rtol = 1e-9 if form == abi.FORM_PLAIN else 2e-6
    for k, v in ref.items():
        # signed sums (momentum, force) nearly cancel: their summation order
        # alone moves them by ~1e-16 of the sum of |terms|
        np.testing.assert_allclose(dev[k], v, rtol=rtol, atol=1e-8, err_msg=k)


def test_probe_matches_host_shepard_sum():
    p, arr = load(cases.dam_break_water(dx=0.02))
    pts = np.array([[0.5, 0.5], [0.3, 1.5], [0.95, 0.2], [-5.0, 1.0]], np.float32)  # last: outside the grid
    with S.Simulation(p) as g:
        g.upload(arr)
        g.step(20)
        got = g.probe(pts)
        st = g.download()
    x = st["fluid_position"].astype(np.float64)
    R2 = float(np.float32(p.impact_distance_square))
    h2inv = float(np.float32(p.smoothing_length_inverse_square))
    c1, c2, c32 = (float(np.float32(v)) for v in (p.kernel_coefficient_1, p.kernel_coefficient_2,
                                                  p.coefficient_3d_to_2d))
    for k, q in enumerate(pts[:3]):
        r2 = np.sum((x - q.astype(np.float64)) ** 2, axis=1)
        near = r2 < R2
        assert near.sum() > 10  # inside the water column
        w = (np.exp(-r2[near] * h2inv) - c1) * c2 * c32
        ref = [np.sum(st["fluid_velocity"][near, 0] * w) / w.sum(), np.sum(st["fluid_velocity"][near, 1] * w) / w.sum(),
               np.sum(st["fluid_pressure"][near] * w) / w.sum(), np.sum(st["fluid_density"][near] * w) / w.sum()]
        np.testing.assert_allclose(got[k], ref, rtol=1e-4, atol=1e-6 * (1 + np.abs(ref).max()))
    # outside the grid: no neighbours
    np.testing.assert_array_equal(got[3], [0, 0, 0, np.float32(p.reference_density[0])])
