"""Synthetic case generators in the reference's case format.

Each generator returns a Case: the ini keys of config/input.ini and the
particle arrays of data/fluid_particle.dat, solid_particle.dat and
virt_particle.dat, laid out as the reference's own generators lay them out
(lattice at (i + 1/2) dx, virtual wall layers around the tank, cases/*/
particle_generate.cpp).  Case.write() produces a directory the reference
binary and this library both read; Case.params() builds the parameters
without writing particle files (large cases).

Workloads (sizes as the benchmark configurations state them):
  dam_break_water   1.0 x 2.0 m water column in a 4.0 x 3.0 m tank,
                    dx = 0.02 (5,000 fluid), 3 wall layers, 2,000 steps
  beam              0.2 x 0.02 m cantilever + 0.06 m clamp, dx = 0.001
                    (5,200 solid), first bending mode, tip speed 0.01 c_s
  gate              hydroelastic gate: 0.1 x 0.14 m water, 0.005 x 0.079 m
                    rubber gate, air in a 0.6 x 0.3 m tank, dx = 0.0005
  dam_break_gas     dam break with air, dx = 0.0017 (~4.15M fluid)
The smoothing kernel is the reference's truncated Gaussian with h = 1.2 dx
(kernel.cpp:25-41 is its only kernel; C32 is tuned for h/d = 1.2).
"""
from __future__ import annotations

import math
import os
import tempfile
from dataclasses import dataclass, field
from pathlib import Path

import numpy as np

from . import abi

G = 9.81


@dataclass
class Case:
    name: str
    ini: dict
    fluid_position: np.ndarray = None   # (n, 2) f32
    fluid_velocity: np.ndarray = None
    fluid_density: np.ndarray = None    # (n,) f32
    fluid_pressure: np.ndarray = None
    fluid_phase: np.ndarray = None      # (n,) i32, liquid first
    solid_position: np.ndarray = None   # (n, 2) f64
    solid_velocity: np.ndarray = None
    solid_reference_position: np.ndarray = None
    solid_material_type: np.ndarray = None
    solid_boundary_type: np.ndarray = None
    virt_position: np.ndarray = None    # (n, 2) f32
    virt_boundary_type: np.ndarray = None
    notes: dict = field(default_factory=dict)

    # ---- counts ------------------------------------------------------------
    @property
    def n_liquid(self):
        return int(np.sum(self.fluid_phase == abi.LIQUID)) if self.fluid_phase is not None else 0

    @property
    def n_gas(self):
        return int(np.sum(self.fluid_phase == abi.GAS)) if self.fluid_phase is not None else 0

    @property
    def n_fluid(self):
        return 0 if self.fluid_phase is None else len(self.fluid_phase)

    @property
    def n_solid(self):
        return 0 if self.solid_position is None else len(self.solid_position)

    @property
    def n_virt(self):
        return 0 if self.virt_position is None else len(self.virt_position)

    def arrays(self) -> dict:
        """Host-state arrays for Simulation.upload (the .dat fields)."""
        out = {}
        for k in abi.INPUT_FIELDS:
            v = getattr(self, k)
            if v is not None and len(v):
                out[k] = np.ascontiguousarray(v)
        return out

    # ---- files -------------------------------------------------------------
    def ini_text(self) -> str:
        lines = [f"# {self.name}: generated by sphnj_gb300.cases"]
        for k, v in self.ini.items():
            lines.append(f"{k} = {v}")
        return "\n".join(lines) + "\n"

    def write(self, root) -> Path:
        root = Path(root)
        (root / "config").mkdir(parents=True, exist_ok=True)
        (root / "data").mkdir(parents=True, exist_ok=True)
        (root / "config" / "input.ini").write_text(self.ini_text())
        d = root / "data"
        with open(d / "fluid_particle.dat", "w") as f:
            f.write(f"{self.n_liquid} {self.n_gas}\n")
            if self.n_fluid:
                cols = np.column_stack([self.fluid_position, self.fluid_velocity, self.fluid_density,
                                        self.fluid_pressure]).astype(np.float32)
                body = np.column_stack([cols.astype(np.float64), self.fluid_phase.astype(np.float64)])
                np.savetxt(f, body, fmt=["%.9g"] * 6 + ["%d"])
        with open(d / "solid_particle.dat", "w") as f:
            f.write(f"{self.n_solid}\n")
            if self.n_solid:
                body = np.column_stack([self.solid_position, self.solid_velocity, self.solid_reference_position,
                                        self.solid_material_type, self.solid_boundary_type])
                np.savetxt(f, body, fmt=["%.17g"] * 6 + ["%d", "%d"])
        with open(d / "virt_particle.dat", "w") as f:
            f.write(f"{self.n_virt}\n")
            if self.n_virt:
                body = np.column_stack([self.virt_position.astype(np.float64), self.virt_boundary_type])
                np.savetxt(f, body, fmt=["%.9g", "%.9g", "%d"])
        return root

    def params(self) -> abi.Params:
        """Params from this case's ini keys and particle counts (reads only the
        ini through the library; particle files are not written)."""
        from . import derive, read_ini

        with tempfile.TemporaryDirectory() as t:
            ini = Path(t) / "input.ini"
            ini.write_text(self.ini_text())
            p, rc = read_ini(ini)
        if rc:
            raise ValueError(f"{self.name}: ini rejected ({rc})")
        p.fluid_number[0] = self.n_liquid
        p.fluid_number[1] = self.n_gas
        p.fluid_number_total = self.n_fluid
        p.solid_number = self.n_solid
        p.virt_number = self.n_virt
        return derive(p)


def _fmt(x) -> str:
    if isinstance(x, bool):
        return "true" if x else "false"
    if isinstance(x, (int, np.integer)):
        return str(int(x))
    return repr(float(x))


def base_ini(dx, h_ratio=1.2, dt=1e-4, iend=2000, **kw) -> dict:
    ini = dict(
        gravity=G, is_steady=False,
        particle_shift_coef=1.0, is_viscid=False, min_pressure=-1.013e5,
        liquid_density=1000.0, liquid_sound_speed=20.0, liquid_gamma=7.0, liquid_viscosity=1.01e-3,
        gas_density=1.0, gas_sound_speed=20.0, gas_gamma=1.4, gas_viscosity=17.9e-6,
        solid_density=2700.0, youngs_modulus=67.5e9, poisson_ratio=0.34,
        arti_vis_alpha=2.5, arti_vis_beta=2.5, solid_fixed_speed_x=0.0, solid_fixed_speed_y=0.0,
        is_2D_strain=False, is_plastic=False,
        auxetic_density=636.0, auxetic_modulus=2.0e8, auxetic_poisson_ratio=-0.2,
        yield_strain=0.0, yield_stress=0.7e7, harden_strain=0.5, harden_coef=100.0,
        cell_xmin=0.0, cell_xmax=1.0, cell_ymin=0.0, cell_ymax=1.0,
        domain_xmin=0.0, domain_xmax=1.0, domain_ymin=0.0, domain_ymax=1.0,
        dt=dt, istart=0, iend=iend, result_interval=100, sort_every_step=50, solid_sub_step=1,
        shift_per_step=10,
        smoothing_length=h_ratio * dx, particle_diameter=dx, impact_length_hsml_ratio=3.0, thread_num=32,
    )
    ini.update(kw)
    return {k: _fmt(v) for k, v in ini.items()}


def _eos_density(p, rho0, c, gamma):
    """pressureToDensity (fluid.cu:6-13)."""
    return rho0 * np.power(p * gamma / (rho0 * c * c) + 1.0, 1.0 / gamma)


def tank(name, dx, tank_w, tank_h, col_w, col_h, layers=3, gas=False, rho_l=1000.0, rho_g=1.0, c=None,
         c_gas=None, h_ratio=1.2, cfl=0.13, iend=2000, shift_per_step=10, jitter=0.0, seed=0, closed_top=True,
         extra_ini=None, solid=None) -> Case:
    """Water column in a walled tank, optionally with air (the reference's
    dam_break generator layout, cases/dam_break/particle_generate.cpp:55-114).

    solid: optional (position, velocity, reference, material, boundary) arrays
    of solid particles; fluid lattice sites inside the solid's bounding boxes
    given in solid['exclude'] are left empty."""
    if c is None:
        c = 10.0 * math.sqrt(2.0 * G * col_h)
    if c_gas is None:
        c_gas = c
    nx = int(round(tank_w / dx))
    ny = int(round(tank_h / dx))
    L = layers
    ii, jj = np.meshgrid(np.arange(-L, nx + L), np.arange(-L, ny + L if closed_top else ny), indexing="ij")
    ii = ii.ravel()
    jj = jj.ravel()
    x = (ii + 0.5) * dx
    y = (jj + 0.5) * dx
    if jitter:
        rng = np.random.default_rng(seed)
        x = x + rng.uniform(-jitter, jitter, x.shape) * dx
        y = y + rng.uniform(-jitter, jitter, y.shape) * dx
    outside = (ii < 0) | (ii >= nx) | (jj < 0) | (jj >= ny)
    liquid = ~outside & (ii < int(round(col_w / dx))) & (jj < int(round(col_h / dx)))
    gas_m = ~outside & ~liquid if gas else np.zeros_like(liquid)
    if solid is not None:
        for (x0, x1, y0, y1) in solid.get("exclude", []):
            inside = (x > x0) & (x < x1) & (y > y0) & (y < y1)
            liquid &= ~inside
            gas_m &= ~inside
            outside &= ~inside
    # liquid particles first, then gas (the header counts liquid then gas)
    fx = np.concatenate([x[liquid], x[gas_m]])
    fy = np.concatenate([y[liquid], y[gas_m]])
    phase = np.concatenate([np.full(liquid.sum(), abi.LIQUID), np.full(gas_m.sum(), abi.GAS)]).astype(np.int32)
    p = np.where(phase == abi.LIQUID, rho_l * G * (col_h - fy), 0.0)
    p = np.maximum(p, 0.0)
    rho = np.where(phase == abi.LIQUID, _eos_density(p, rho_l, c, 7.0), rho_g)
    h = h_ratio * dx
    dt = cfl * h / max(c, c_gas)
    margin = L * dx + 3.0 * h
    ini = base_ini(dx, h_ratio=h_ratio, dt=float(np.float32(dt)), iend=iend, liquid_density=rho_l,
                   liquid_sound_speed=c, gas_density=rho_g, gas_sound_speed=c_gas, shift_per_step=shift_per_step,
                   cell_xmin=-margin, cell_xmax=tank_w + margin, cell_ymin=-margin, cell_ymax=tank_h + margin,
                   domain_xmin=0.0, domain_xmax=tank_w, domain_ymin=0.0, domain_ymax=tank_h)
    if extra_ini:
        ini.update({k: _fmt(v) for k, v in extra_ini.items()})
    case = Case(
        name=name, ini=ini,
        fluid_position=np.column_stack([fx, fy]).astype(np.float32),
        fluid_velocity=np.zeros((len(fx), 2), np.float32),
        fluid_density=rho.astype(np.float32),
        fluid_pressure=p.astype(np.float32),
        fluid_phase=phase,
        virt_position=np.column_stack([x[outside], y[outside]]).astype(np.float32),
        virt_boundary_type=np.full(int(outside.sum()), abi.SLIP, np.int32),
        notes=dict(dx=dx, c=c, tank=(tank_w, tank_h), column=(col_w, col_h), layers=layers),
    )
    if solid is not None:
        case.solid_position = solid["position"]
        case.solid_velocity = solid["velocity"]
        case.solid_reference_position = solid["reference"]
        case.solid_material_type = solid["material"]
        case.solid_boundary_type = solid["boundary"]
    return case


def dam_break_water(dx=0.02, iend=2000, layers=3, **kw) -> Case:
    """Plain 2-D dam break, water only: 1.0 x 2.0 m column, 4.0 x 3.0 m tank."""
    return tank("dam_break_water", dx, 4.0, 3.0, 1.0, 2.0, layers=layers, gas=False, iend=iend, **kw)


def dam_break_gas(dx=0.0017, iend=20000, layers=3, **kw) -> Case:
    """Gas-liquid dam break: the same geometry with air (rho = 1.0) in the rest
    of the tank (dx = 0.0017 gives ~0.69M water + ~3.46M air)."""
    return tank("dam_break_gas", dx, 4.0, 3.0, 1.0, 2.0, layers=layers, gas=True, iend=iend, **kw)


def beam(dx=0.001, length=0.2, thick=0.02, clamp=0.06, E=1.4e6, nu=0.4, rho=1000.0, amp=0.01, h_ratio=1.2,
         cfl=0.1, iend=2000, material=abi.LINEAR_ELASTIC, jitter=0.0, seed=0, extra_ini=None) -> Case:
    """Cantilever clamped over `clamp` at its left end (FIXED particles),
    initial transverse velocity from the first bending mode (kL = 1.875) with
    tip speed amp * c_s (same form as cases/beam_vibrate/particle_generate.cpp:
    55-74)."""
    nL = int(round(length / dx))
    nC = int(round(clamp / dx))
    nT = int(round(thick / dx))
    ii, jj = np.meshgrid(np.arange(-nC, nL), np.arange(nT), indexing="ij")
    ii = ii.ravel()
    jj = jj.ravel()
    x = (ii + 0.5) * dx
    y = (jj + 0.5) * dx - 0.5 * thick
    if jitter:
        rng = np.random.default_rng(seed)
        x = x + rng.uniform(-jitter, jitter, x.shape) * dx
        y = y + rng.uniform(-jitter, jitter, y.shape) * dx
    K = E / (3.0 * (1.0 - 2.0 * nu))
    cs = math.sqrt(K / rho)
    kl = 1.875

    def shape(z):
        k = kl / length
        return ((math.cos(kl) + math.cosh(kl)) * (np.cosh(k * z) - np.cos(k * z))
                + (math.sin(kl) - math.sinh(kl)) * (np.sinh(k * z) - np.sin(k * z)))

    fixed = ii < 0
    vy = np.where(fixed, 0.0, amp * cs * shape(np.maximum(x, 0.0)) / shape(np.array(length)))
    h = h_ratio * dx
    dt = cfl * h / cs
    defl = amp * cs / ((kl / length) ** 2 * math.sqrt(E * thick ** 2 / (12 * rho))) * 2.0 + 3 * h
    ini = base_ini(dx, h_ratio=h_ratio, dt=float(np.float32(dt)), iend=iend, gravity=0.0,
                   solid_density=rho, youngs_modulus=E, poisson_ratio=nu, shift_per_step=1,
                   cell_xmin=-clamp - 4 * h, cell_xmax=length + 4 * h + defl,
                   cell_ymin=-0.5 * thick - defl - 4 * h, cell_ymax=0.5 * thick + defl + 4 * h,
                   domain_xmin=-clamp, domain_xmax=length + defl, domain_ymin=-defl, domain_ymax=defl)
    if extra_ini:
        ini.update({k: _fmt(v) for k, v in extra_ini.items()})
    pos = np.column_stack([x, y]).astype(np.float64)
    return Case(
        name="beam", ini=ini,
        solid_position=pos.copy(), solid_velocity=np.column_stack([np.zeros_like(vy), vy]),
        solid_reference_position=pos.copy(),
        solid_material_type=np.full(len(x), material, np.int32),
        solid_boundary_type=np.where(fixed, abi.FIXED, abi.UNCONSTRAINED).astype(np.int32),
        notes=dict(dx=dx, cs=cs, length=length, thick=thick, clamp=clamp,
                   omega1=kl * kl * math.sqrt(E * thick ** 2 / (12 * rho)) / length ** 2),
    )


def gate(dx=0.0005, iend=2000, substeps=8, layers=8, gas=True, E=10.0e6, nu=0.4, rho_s=1100.0, **kw) -> Case:
    """Hydroelastic dam break on an elastic gate: water 0.1 x 0.14 m held by a
    0.005 x 0.079 m gate (bottom free, clamped at its top to a rigid wall
    above it), air in the rest of a 0.6 x 0.3 m tank."""
    t = 0.005
    gh = 0.079
    x0 = 0.1
    top = 0.16
    nT = int(round(t / dx))
    nG = int(round(gh / dx))
    nW = int(round((top - gh) / dx))
    ii, jj = np.meshgrid(np.arange(nT), np.arange(nG + nW), indexing="ij")
    ii = ii.ravel()
    jj = jj.ravel()
    sx = x0 + (ii + 0.5) * dx
    sy = (jj + 0.5) * dx
    fixed = jj >= nG
    pos = np.column_stack([sx, sy]).astype(np.float64)
    solid = dict(position=pos.copy(), velocity=np.zeros_like(pos), reference=pos.copy(),
                 material=np.full(len(sx), abi.LINEAR_ELASTIC, np.int32),
                 boundary=np.where(fixed, abi.FIXED, abi.UNCONSTRAINED).astype(np.int32),
                 exclude=[(x0, x0 + t, 0.0, top)])
    K = E / (3.0 * (1.0 - 2.0 * nu))
    cs_s = math.sqrt(K / rho_s)
    c = 10.0 * math.sqrt(2.0 * G * 0.14)
    case = tank("gate", dx, 0.6, 0.3, x0, 0.14, layers=layers, gas=gas, iend=iend, solid=solid,
                extra_ini=dict(solid_density=rho_s, youngs_modulus=E, poisson_ratio=nu, solid_sub_step=substeps,
                               is_2D_strain=False), **kw)
    # the solid time step is dt / substeps: check it resolves the solid sound speed
    case.notes.update(cs_solid=cs_s, substeps=substeps)
    return case


def auxetic_block(dx=0.002, n=20, rate=1000.0, yield_stress=2.0e6, yield_strain=0.05, rho=200.0, cfl=0.2,
                  iend=200, plastic=True) -> Case:
    """Square block of the reference's AUXETIC (principal-strain plasticity)
    material under uniform compression v = -rate * (x - centre): exercises
    solid.cu:80-148 including the max_strain history."""
    ii, jj = np.meshgrid(np.arange(n), np.arange(n), indexing="ij")
    x = (ii.ravel() + 0.5) * dx
    y = (jj.ravel() + 0.5) * dx
    cx = cy = 0.5 * n * dx
    modulus = yield_stress / yield_strain
    cs = math.sqrt(modulus / rho)
    h = 1.2 * dx
    pos = np.column_stack([x, y]).astype(np.float64)
    vel = np.column_stack([-rate * (x - cx), -rate * (y - cy)])
    L = n * dx
    ini = base_ini(dx, dt=float(np.float32(cfl * h / cs)), iend=iend, gravity=0.0, auxetic_density=rho,
                   yield_stress=yield_stress, yield_strain=yield_strain, is_plastic=plastic, harden_strain=0.3,
                   harden_coef=1.0e9, solid_density=rho, youngs_modulus=modulus, poisson_ratio=0.2,
                   shift_per_step=1, cell_xmin=-L, cell_xmax=2 * L, cell_ymin=-L, cell_ymax=2 * L,
                   domain_xmin=-L, domain_xmax=2 * L, domain_ymin=-L, domain_ymax=2 * L)
    return Case(name="auxetic_block", ini=ini, solid_position=pos.copy(), solid_velocity=vel,
                solid_reference_position=pos.copy(), solid_material_type=np.full(len(x), abi.AUXETIC, np.int32),
                solid_boundary_type=np.zeros(len(x), np.int32), notes=dict(dx=dx, cs=cs))


SWEEP_SCENES = 256


def sweep_scene(seed: int, iend: int = 2000) -> Case:
    """Scene `seed` (0..255) of the batched sweep of independent scenes of
    uneven size, drawn from a per-scene generator seeded with `seed`:
      seeds 0..127    water-only dam breaks: a 1.0 m wide column of height
                      H/W ~ U[0.5, 2.5] in a 4.0 x 3.0 m tank, particle count
                      log-uniform in [2k, 60k] (dx = sqrt(W H / N)), 3 wall
                      layers;
      seeds 128..255  cantilever beams: length L ~ U[0.1, 0.3] m, thickness
                      L/10, clamp 0.3 L, E log-uniform in [0.5, 20] MPa,
                      nu ~ U[0.3, 0.45], rho = 1000, particle count
                      log-uniform in [1k, 20k];
    every lattice jittered by +-0.01 dx."""
    if not 0 <= seed < SWEEP_SCENES:
        raise ValueError(f"sweep scene seed {seed} outside 0..{SWEEP_SCENES - 1}")
    rng = np.random.default_rng(seed)
    if seed < SWEEP_SCENES // 2:
        aspect = rng.uniform(0.5, 2.5)
        n = math.exp(rng.uniform(math.log(2_000), math.log(60_000)))
        col_w, col_h = 1.0, aspect
        dx = math.sqrt(col_w * col_h / n)
        case = tank(f"sweep{seed:03d}_dam", dx, 4.0, 3.0, col_w, col_h, layers=3, gas=False, iend=iend,
                    jitter=0.01, seed=10_000 + seed)
        case.notes.update(kind="dam_break", aspect=aspect, seed=seed)
        return case
    length = rng.uniform(0.1, 0.3)
    E = math.exp(rng.uniform(math.log(0.5e6), math.log(20e6)))
    nu = rng.uniform(0.3, 0.45)
    n = math.exp(rng.uniform(math.log(1_000), math.log(20_000)))
    thick, clamp = 0.1 * length, 0.3 * length
    dx = math.sqrt((length + clamp) * thick / n)
    case = beam(dx=dx, length=length, thick=thick, clamp=clamp, E=E, nu=nu, rho=1000.0, iend=iend,
                jitter=0.01, seed=10_000 + seed)
    case.name = f"sweep{seed:03d}_beam"
    case.notes.update(kind="beam", E=E, nu=nu, seed=seed)
    return case


def by_name(name: str, **kw) -> Case:
    return {"dam_break_water": dam_break_water, "dam_break_gas": dam_break_gas, "beam": beam,
            "gate": gate, "auxetic_block": auxetic_block}[name](**kw)
