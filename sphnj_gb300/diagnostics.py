"""Global diagnostics of a downloaded state (host side, float64).

Definitions (the same ones the reference-build harness writes for the golden
fixtures, oracle/ref/harness.cu):
  front    max x over liquid particles + d/2        (outputEdge, output.cu:339-352)
  mom      sum m v,    m = rho0[phase] d^2 (constant particle mass)
  ek       sum m |v|^2 / 2 over fluid
  rho_sum  sum rho d^2
  tip      position - reference position of the solid particle with the
           largest reference x (ties: closest to the mean reference y)
  eks      sum rho_s d^2 |v|^2 / 2 over solid
  eps      sum (lambda/2 tr(E)^2 + mu E:E) d^2, E = (F^T F - I)/2
           (outputTotalEnergy, output.cu:426-455)
"""
from __future__ import annotations

import numpy as np

from . import abi

COLUMNS = ["step", "front", "mom_x", "mom_y", "ek", "rho_sum", "tip_x", "tip_y", "eks", "eps"]


def diagnostics(p: abi.Params, st: dict, step: int = 0) -> np.ndarray:
    d = float(np.float32(p.particle_diameter))
    d2 = d * d
    front = mx = my = ek = rs = 0.0
    if p.fluid_number_total:
        x = st["fluid_position"].astype(np.float64)
        v = st["fluid_velocity"].astype(np.float64)
        ph = st["fluid_phase"]
        rho0 = np.where(ph == abi.GAS, np.float64(np.float32(p.reference_density[1])),
                        np.float64(np.float32(p.reference_density[0])))
        m = rho0 * d2
        liq = ph == abi.LIQUID
        front = (x[liq, 0].max() if liq.any() else -1e300) + 0.5 * np.float64(np.float32(p.particle_diameter))
        mx = float(np.sum(m * v[:, 0]))
        my = float(np.sum(m * v[:, 1]))
        ek = float(np.sum(0.5 * m * np.sum(v * v, axis=1)))
        rs = float(np.sum(st["fluid_density"].astype(np.float64)) * d2)
    tx = ty = eks = eps = 0.0
    if p.solid_number:
        x = st["solid_position"]
        r = st["solid_reference_position"]
        v = st["solid_velocity"]
        F = st["solid_deformation"].reshape(-1, 4)
        ymean = r[:, 1].mean()
        xmax = r[:, 0].max()
        cand = np.nonzero(r[:, 0] >= xmax - 1e-12)[0]
        best = cand[np.argmin(np.abs(r[cand, 1] - ymean))]
        tx, ty = x[best] - r[best]
        rho = float(np.float32(p.solid_reference_density))
        lam, mu = float(np.float32(p.lambda_)), float(np.float32(p.nu))
        eks = float(np.sum(0.5 * rho * d2 * np.sum(v * v, axis=1)))
        f00, f10, f01, f11 = F[:, 0], F[:, 1], F[:, 2], F[:, 3]
        e00 = 0.5 * (f00 * f00 + f10 * f10 - 1.0)
        e11 = 0.5 * (f01 * f01 + f11 * f11 - 1.0)
        e01 = 0.5 * (f00 * f01 + f10 * f11)
        tr = e00 + e11
        eps = float(np.sum((0.5 * lam * tr * tr + mu * (e00 * e00 + e11 * e11 + 2 * e01 * e01)) * d2))
    return np.array([step, front, mx, my, ek, rs, tx, ty, eks, eps])
