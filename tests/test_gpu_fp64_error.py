"""Error of both GPU forms against the FP64 oracle on the benchmark
configurations themselves - the "stated FP64 error" of the metric.

  - the 4.15M-particle gas-liquid dam break (dx 0.0017), both forms against
    the oracle's double-precision build for 60 steps (two sort steps and the
    incremental steps between them);
  - the same geometry at dx 0.0068 (259k particles) for 2,000 steps, and the
    4.15M case for its full 20,000 steps, mixed against plain (long runs);
  - the cantilever at dx 0.001 (5,200 particles) over ten first-mode periods
    (long run);
  - the gas-liquid-solid gate at its configured dx 0.0005 (~720k particles,
    k = 8 solid sub-steps) against the FP64 oracle over a window, and mixed
    against plain over the run (long run);
  - a subset of the 256-scene sweep batched in the mixed form against the
    FP64 oracle scene by scene.

Particles are permuted by every sort (a stable sort by cell id), and runs
that differ in rounding can put a particle near a cell boundary into
different cells, so per-particle positions are compared only between sorts
(step 50, before the second sort, after checking that both runs sorted alike
at step 1); other comparisons use permutation-free quantities: the surge
front (max x of liquid + d/2, outputEdge, output.cu:339-352), mass
sum rho d^2, kinetic and potential energy, momentum, the sorted x and y
coordinates of the liquid (largest gap, in particle spacings) and, for
solids, the tip displacement (the solid particle with the largest reference
x; for the gate the free end: smallest reference y).

With SPHNJ_RECORD_DIR set each test writes its measured errors as
fp64_<name>.json (committed under tests/records/; bench.py reports them).
The long runs (minutes) run with SPHNJ_LONG=1.
"""
from __future__ import annotations

import os

import numpy as np
import pytest

import oracle
import sphnj_gb300 as S
from sphnj_gb300 import abi, cases

from helpers import record

pytestmark = [pytest.mark.gpu, pytest.mark.slow]

LONG = os.environ.get("SPHNJ_LONG") == "1"
long_run = pytest.mark.skipif(not LONG, reason="long run (minutes): SPHNJ_LONG=1; its record is in tests/records")

PLAIN, MIXED = abi.FORM_PLAIN, abi.FORM_MIXED
FLUID_MASK = abi.F_FLUID_KINEMATICS | abi.F_FLUID_THERMO
SOLID_MASK = abi.F_SOLID_KINEMATICS | abi.F_SOLID_DERIVED


def fluid_summary(p, st) -> dict:
    """Permutation-free fluid quantities of a state, in float64."""
    d = float(np.float32(p.particle_diameter))
    x = st["fluid_position"].astype(np.float64)
    v = st["fluid_velocity"].astype(np.float64)
    ph = st["fluid_phase"]
    rho0 = np.where(ph == abi.GAS, float(np.float32(p.reference_density[1])),
                    float(np.float32(p.reference_density[0])))
    m = rho0 * d * d
    liq = ph == abi.LIQUID
    g = -float(np.float32(p.gravity[1]))
    return {
        "front": float(x[liq, 0].max() + 0.5 * d) if liq.any() else float("nan"),
        "mass": float(np.sum(st["fluid_density"].astype(np.float64)) * d * d),
        "kinetic": float(np.sum(0.5 * m * np.sum(v * v, axis=1))),
        "potential": float(np.sum(m * g * x[:, 1])),
        "mom_x": float(np.sum(m * v[:, 0])),
        "mom_y": float(np.sum(m * v[:, 1])),
        "_xs": np.sort(x[liq, 0]), "_ys": np.sort(x[liq, 1]),
    }


def fluid_compare(a: dict, ref: dict, dx: float, scales: dict) -> dict:
    """Errors of summary a against ref: relative to the given scales, and the
    largest gap of the sorted liquid coordinates in particle spacings."""
    out = {k: abs(a[k] - ref[k]) / scales[k] for k in ("front", "mass", "kinetic", "potential", "mom_x", "mom_y")}
    out["sorted_x_spacings"] = float(np.max(np.abs(a["_xs"] - ref["_xs"]))) / dx
    out["sorted_y_spacings"] = float(np.max(np.abs(a["_ys"] - ref["_ys"]))) / dx
    return out


def public(s: dict) -> dict:
    return {k: v for k, v in s.items() if not k.startswith("_")}


def worst_of(rows: list) -> dict:
    out = {}
    for r in rows:
        for k, v in r.items():
            out[k] = max(out.get(k, 0.0), v)
    return out


def gpu_sim(p, arr, form):
    g = S.Simulation(p, form)
    g.upload(arr)
    return g


def fp64_sim(p, arr):
    o = oracle.OracleSim(p, oracle.FP64, threads=0)
    o.upload(arr)
    return o


# ---- the benchmark's 4.15M dam break ----------------------------------------

@pytest.fixture(scope="module")
def headline():
    case = cases.dam_break_gas(dx=0.0017)
    p = case.params()
    arr = case.arrays()
    # wall normals once (device nine-way merge), given to every run
    with S.Simulation(p) as g:
        g.upload(arr)
        arr["virt_normal"] = np.ascontiguousarray(g.download(abi.F_VIRT)["virt_normal"])
    return case, p, arr


def test_headline_both_forms_against_fp64_oracle(headline):
    """4.15M particles, 60 steps (sorts at steps 1 and 51): per-particle
    positions at step 50 in particle spacings, and the permutation-free
    quantities at steps 1, 50 and 60, for the mixed and the plain form."""
    case, p, arr = headline
    dx = float(p.particle_diameter)
    marks = [1, 50, 60]
    runs = {"plain": PLAIN, "mixed": MIXED}
    states = {}
    for name, form in runs.items():
        with S.Simulation(p, form) as g:
            g.upload(arr)
            done, st = 0, {}
            for m in marks:
                g.step(m - done)
                done = m
                s = g.download(FLUID_MASK | abi.F_CELL_IDS)
                st[m] = {"summary": fluid_summary(p, s), "cell": s["fluid_cell_id"].copy() if m == 1 else None,
                         "pos": s["fluid_position"].copy() if m == 50 else None}
            states[name] = st
    o = fp64_sim(p, arr)
    ref, done = {}, 0
    try:
        for m in marks:
            o.step(m - done)
            done = m
            s = o.download(FLUID_MASK | abi.F_CELL_IDS)
            ref[m] = {"summary": fluid_summary(p, s), "cell": s["fluid_cell_id"].copy() if m == 1 else None,
                      "pos": s["fluid_position"].copy() if m == 50 else None}
    finally:
        o.close()
    s0 = ref[marks[-1]]["summary"]
    scales = {"front": s0["front"], "mass": s0["mass"], "kinetic": max(s0["kinetic"], 1e-30),
              "potential": abs(s0["potential"]), "mom_x": max(abs(s0["mom_x"]), abs(s0["mom_y"]), 1e-30),
              "mom_y": max(abs(s0["mom_x"]), abs(s0["mom_y"]), 1e-30)}
    summary = {}
    for name in runs:
        # the first sort ran on identical inputs: same ids, same permutation
        assert np.array_equal(states[name][1]["cell"], ref[1]["cell"]), name
        dpos = np.abs(states[name][50]["pos"].astype(np.float64) - ref[50]["pos"]).max(axis=1) / dx
        per_mark = {m: fluid_compare(states[name][m]["summary"], ref[m]["summary"], dx, scales) for m in marks}
        summary[name] = dict(worst_of(list(per_mark.values())), position_max_spacings_step50=float(dpos.max()),
                             position_rms_spacings_step50=float(np.sqrt(np.mean(dpos ** 2))))
    record("fp64_dam_break_gas_4M_60_steps", {
        "case": "gas-liquid dam break, dx 0.0017", "particles": int(p.fluid_number_total), "steps": marks[-1],
        "compared_at": marks, "reference": "oracle, double precision", "summary": summary,
        "fp64_at_last": public(s0)})
    print({k: {q: f"{w:.2e}" for q, w in v.items()} for k, v in summary.items()})
    for name in runs:
        assert summary[name]["position_max_spacings_step50"] < 1e-2, (name, summary[name])
        assert summary[name]["front"] < 5e-3 and summary[name]["mass"] < 1e-4, (name, summary[name])


@long_run
def test_dam_break_2000_steps_against_fp64_oracle():
    """The benchmark geometry at dx 0.0068 (259k particles), 2,000 steps
    sampled every 200: front, mass, energy and momentum of both forms against
    the FP64 oracle, and each run's drift of mass and mechanical energy from
    its start."""
    case = cases.dam_break_gas(dx=0.0068)
    p = case.params()
    arr = case.arrays()
    with S.Simulation(p) as g:
        g.upload(arr)
        arr["virt_normal"] = np.ascontiguousarray(g.download(abi.F_VIRT)["virt_normal"])
    dx = float(p.particle_diameter)
    every, steps = 200, 2000
    traj = {}
    for name, form in (("plain", PLAIN), ("mixed", MIXED)):
        with gpu_sim(p, arr, form) as g:
            rows = [fluid_summary(p, g.download(FLUID_MASK))]
            for _ in range(steps // every):
                g.step(every)
                rows.append(fluid_summary(p, g.download(FLUID_MASK)))
        traj[name] = rows
    o = fp64_sim(p, arr)
    try:
        rows = [fluid_summary(p, o.download(FLUID_MASK))]
        for _ in range(steps // every):
            o.step(every)
            rows.append(fluid_summary(p, o.download(FLUID_MASK)))
    finally:
        o.close()
    traj["fp64"] = rows
    s0 = rows[-1]
    scales = {"front": s0["front"], "mass": s0["mass"], "kinetic": s0["kinetic"], "potential": abs(s0["potential"]),
              "mom_x": max(abs(s0["mom_x"]), abs(s0["mom_y"])), "mom_y": max(abs(s0["mom_x"]), abs(s0["mom_y"]))}
    summary, drift = {}, {}
    for name in ("plain", "mixed"):
        summary[name] = worst_of([fluid_compare(a, b, dx, scales) for a, b in zip(traj[name], rows)])
    for name in ("plain", "mixed", "fp64"):
        t = traj[name]
        e0 = t[0]["kinetic"] + t[0]["potential"]
        drift[name] = {"mass": (t[-1]["mass"] - t[0]["mass"]) / t[0]["mass"],
                       "mechanical_energy": (t[-1]["kinetic"] + t[-1]["potential"] - e0) / abs(e0)}
    record("fp64_dam_break_gas_259k_2000_steps", {
        "case": "gas-liquid dam break, dx 0.0068", "particles": int(p.fluid_number_total), "steps": steps,
        "every": every, "reference": "oracle, double precision", "summary": summary, "drift": drift,
        "front_fp64": [r["front"] for r in rows], "front_mixed": [r["front"] for r in traj["mixed"]],
        "front_plain": [r["front"] for r in traj["plain"]]})
    print(summary, drift)
    for name in ("plain", "mixed"):
        assert summary[name]["front"] < 5e-3, (name, summary[name])
        assert summary[name]["mass"] < 1e-3, (name, summary[name])


@long_run
def test_headline_20000_steps_mixed_against_plain(headline):
    """The 4.15M case for its configured 20,000 steps on the GPU (the FP64
    oracle would take hours): front, mass and energy of the mixed form
    against the plain form every 2,000 steps, and each form's drift."""
    case, p, arr = headline
    every, steps = 2000, 20000
    traj = {}
    for name, form in (("plain", PLAIN), ("mixed", MIXED)):
        with gpu_sim(p, arr, form) as g:
            rows = [fluid_summary(p, g.download(FLUID_MASK))]
            for _ in range(steps // every):
                g.step(every)
                rows.append(fluid_summary(p, g.download(FLUID_MASK)))
            g.synchronize()
        traj[name] = rows
    dx = float(p.particle_diameter)
    ref = traj["plain"]
    s0 = ref[-1]
    scales = {"front": s0["front"], "mass": s0["mass"], "kinetic": s0["kinetic"], "potential": abs(s0["potential"]),
              "mom_x": max(abs(s0["mom_x"]), abs(s0["mom_y"])), "mom_y": max(abs(s0["mom_x"]), abs(s0["mom_y"]))}
    diff = worst_of([fluid_compare(a, b, dx, scales) for a, b in zip(traj["mixed"], ref)])
    drift = {}
    for name, t in traj.items():
        e0 = t[0]["kinetic"] + t[0]["potential"]
        drift[name] = {"mass": (t[-1]["mass"] - t[0]["mass"]) / t[0]["mass"],
                       "mechanical_energy": (t[-1]["kinetic"] + t[-1]["potential"] - e0) / abs(e0)}
    record("fp64_dam_break_gas_4M_20000_steps", {
        "case": "gas-liquid dam break, dx 0.0017", "particles": int(p.fluid_number_total), "steps": steps,
        "every": every, "summary": {"mixed_vs_plain": diff}, "drift": drift,
        "front_mixed": [r["front"] for r in traj["mixed"]], "front_plain": [r["front"] for r in ref]})
    print(diff, drift)
    assert diff["front"] < 5e-3 and diff["mass"] < 1e-3, diff


# ---- the cantilever (solid only) ---------------------------------------------

def tip_series(sim, every, n):
    """Tip displacement (step, x, y) every `every` steps from the device
    diagnostics (the solid particle with the largest reference x)."""
    out = []
    for _ in range(n):
        sim.step(every)
        dg = sim.diagnostics()
        out.append((dg["step"], dg["tip_disp"][0], dg["tip_disp"][1]))
    return np.array(out)


def zero_crossings(t, y):
    return [t[k] - y[k] * (t[k + 1] - t[k]) / (y[k + 1] - y[k])
            for k in range(len(y) - 1) if y[k] != 0 and np.sign(y[k]) != np.sign(y[k + 1])]


def cantilever(periods: float, every: int):
    case = cases.beam(dx=0.001, cfl=0.25)
    p = case.params()
    arr = case.arrays()
    period = 2 * np.pi / case.notes["omega1"]
    n = int(periods * period / float(p.dt) / every)
    series = {}
    for name, form in (("plain", PLAIN), ("mixed", MIXED)):
        with gpu_sim(p, arr, form) as g:
            series[name] = tip_series(g, every, n)
    o = fp64_sim(p, arr)
    rows = []
    try:
        from sphnj_gb300.diagnostics import COLUMNS, diagnostics

        for _ in range(n):
            o.step(every)
            d = diagnostics(p, o.download(SOLID_MASK), o.step_index)
            rows.append((o.step_index, d[COLUMNS.index("tip_x")], d[COLUMNS.index("tip_y")]))
    finally:
        o.close()
    series["fp64"] = np.array(rows)
    amp = float(np.abs(series["fp64"][:, 2]).max())
    out = {"amplitude_m": amp, "euler_bernoulli_period_s": period, "steps": int(n * every), "every": every,
           "dt": float(p.dt), "particles": int(p.solid_number)}
    for name, s in series.items():
        t = s[:, 0] * float(p.dt)
        cr = zero_crossings(t, s[:, 2])
        out[f"period_{name}_s"] = float(2 * np.mean(np.diff(cr))) if len(cr) >= 2 else None
        if name != "fp64":
            out[f"tip_error_{name}_of_amplitude"] = float(np.abs(s[:, 2] - series["fp64"][:, 2]).max() / amp)
    for name in ("plain", "mixed"):
        if out[f"period_{name}_s"] and out["period_fp64_s"]:
            out[f"period_error_{name}"] = abs(out[f"period_{name}_s"] / out["period_fp64_s"] - 1.0)
    return out, series


def test_cantilever_half_period_against_fp64_oracle():
    """The cantilever at its configured dx 0.001 (5,200 particles) over half
    a first-mode period (out to the largest deflection and back): tip
    displacement of both forms within 0.5% of the FP64 oracle's amplitude."""
    out, _ = cantilever(0.5, 500)
    print(out)
    assert out["tip_error_mixed_of_amplitude"] < 5e-3 and out["tip_error_plain_of_amplitude"] < 5e-3, out


@long_run
def test_cantilever_ten_periods_against_fp64_oracle():
    """Ten first-mode periods (~530k steps): tip displacement and period of
    both forms against the FP64 oracle."""
    out, series = cantilever(10.0, 1000)
    record("fp64_cantilever_10_periods", {"case": "cantilever, dx 0.001, E 1.4 MPa, nu 0.4", "summary": out,
                                          "tip_y_fp64": series["fp64"][:, 2].tolist(),
                                          "tip_y_mixed": series["mixed"][:, 2].tolist(),
                                          "tip_y_plain": series["plain"][:, 2].tolist()})
    print(out)
    assert out["tip_error_mixed_of_amplitude"] < 5e-3, out
    assert out["period_error_mixed"] < 5e-3 and out["period_error_plain"] < 5e-3, out


# ---- the gas-liquid-solid gate -------------------------------------------------

def gate_tip_index(st) -> int:
    """The gate's free end: the solid particle with the smallest reference y,
    closest to the gate's mean reference x."""
    r = st["solid_reference_position"]
    low = np.nonzero(r[:, 1] <= r[:, 1].min() + 1e-12)[0]
    return int(low[np.argmin(np.abs(r[low, 0] - r[:, 0].mean()))])


def gate_tip(st) -> tuple:
    k = gate_tip_index(st)
    d = st["solid_position"][k] - st["solid_reference_position"][k]
    return float(d[0]), float(d[1])


@long_run
def test_gate_at_config_size_against_fp64_oracle():
    """The hydroelastic gate at its configured size: dx 0.0005 (~56k water,
    ~660k air at 1000:1, ~1.6k gate particles, 8 wall layers), k = 8 solid
    sub-steps.  Gate-tip displacement against time over 21,000 steps
    (~0.1 s) for both forms, and over the first 300 steps against the FP64
    oracle together with the fluid's permutation-free quantities."""
    case = cases.gate(dx=0.0005, gas=True, layers=8, substeps=8)
    p = case.params()
    arr = case.arrays()
    with S.Simulation(p) as g:
        g.upload(arr)
        arr["virt_normal"] = np.ascontiguousarray(g.download(abi.F_VIRT)["virt_normal"])
    dx = float(p.particle_diameter)
    every, steps, window = 300, 21000, 300
    tips, fluid = {}, {}
    for name, form in (("plain", PLAIN), ("mixed", MIXED)):
        with gpu_sim(p, arr, form) as g:
            rows = []
            for k in range(steps // every):
                g.step(every)
                st = g.download(SOLID_MASK | (FLUID_MASK if k == 0 else 0))
                if k == 0:
                    fluid[name] = fluid_summary(p, st)
                rows.append((g.step_index,) + gate_tip(st))
            g.synchronize()
        tips[name] = np.array(rows)
    o = fp64_sim(p, arr)
    try:
        o.step(window)
        st = o.download(SOLID_MASK | FLUID_MASK)
        ref_tip = gate_tip(st)
        ref_fluid = fluid_summary(p, st)
    finally:
        o.close()
    amp = float(np.abs(tips["plain"][:, 1:]).max())
    s0 = ref_fluid
    scales = {"front": s0["front"], "mass": s0["mass"], "kinetic": s0["kinetic"], "potential": abs(s0["potential"]),
              "mom_x": max(abs(s0["mom_x"]), abs(s0["mom_y"])), "mom_y": max(abs(s0["mom_x"]), abs(s0["mom_y"]))}
    summary = {"particles": {"fluid": int(p.fluid_number_total), "liquid": int(p.fluid_number[0]),
                             "solid": int(p.solid_number), "virtual": int(p.virt_number)},
               "tip_amplitude_m": amp, "steps": steps, "dt": float(p.dt), "solid_sub_step": int(p.solid_sub_step)}
    for name in ("plain", "mixed"):
        t = tips[name][0]
        tip_err = max(abs(t[1] - ref_tip[0]), abs(t[2] - ref_tip[1]))
        summary[name] = dict(fluid_compare(fluid[name], ref_fluid, dx, scales),
                             tip_error_at_window_m=tip_err)
    summary["mixed_vs_plain_tip_of_amplitude"] = float(np.abs(tips["mixed"][:, 1:] - tips["plain"][:, 1:]).max()
                                                       / max(amp, 1e-30))
    record("fp64_gate_air_config_size", {
        "case": "hydroelastic gate with air, dx 0.0005", "window_vs_fp64_steps": window, "summary": summary,
        "tip_time_s": (tips["plain"][:, 0] * float(p.dt)).tolist(), "tip_plain_m": tips["plain"][:, 1:].tolist(),
        "tip_mixed_m": tips["mixed"][:, 1:].tolist(), "tip_fp64_at_window_m": list(ref_tip)})
    print(summary)
    for name in ("plain", "mixed"):
        assert summary[name]["front"] < 5e-3 and summary[name]["mass"] < 1e-4, summary
    assert summary["mixed_vs_plain_tip_of_amplitude"] < 0.05, summary


# ---- the 256-scene sweep --------------------------------------------------------

SWEEP_SUBSET = [0, 37, 64, 101, 128, 150, 200, 255]


def test_sweep_scenes_batched_mixed_against_fp64_oracle():
    """Eight scenes of the 256-scene sweep (four dam breaks, four beams of
    uneven sizes), advanced together as one batch in the mixed form for 200
    steps, each against the FP64 oracle stepping it alone: front and mass of
    the dam breaks, tip displacement of the beams."""
    loaded = []
    for s in SWEEP_SUBSET:
        c = cases.sweep_scene(s)
        loaded.append((s, c, c.params(), c.arrays()))
    steps = 200
    sims = [S.Simulation(p, MIXED) for _, _, p, _ in loaded]
    try:
        for sim, (_, _, _, arr) in zip(sims, loaded):
            sim.upload(arr)
        with S.Batch(sims) as b:
            b.step(steps)
            b.synchronize()
        got = [sim.download(FLUID_MASK | SOLID_MASK) for sim in sims]
        normals = [sim.download(abi.F_VIRT) for sim in sims]
    finally:
        for sim in sims:
            sim.close()
    rows = {}
    for (seed, c, p, arr), st, nv in zip(loaded, got, normals):
        a = dict(arr)
        if p.virt_number:
            a["virt_normal"] = np.ascontiguousarray(nv["virt_normal"])
        o = fp64_sim(p, a)
        try:
            o.step(steps)
            ref = o.download(FLUID_MASK | SOLID_MASK)
        finally:
            o.close()
        if p.fluid_number_total:
            ga, gb = fluid_summary(p, st), fluid_summary(p, ref)
            rows[seed] = {"kind": "dam_break", "particles": int(p.fluid_number_total),
                          "front": abs(ga["front"] - gb["front"]) / gb["front"],
                          "mass": abs(ga["mass"] - gb["mass"]) / gb["mass"]}
        else:
            from sphnj_gb300.diagnostics import COLUMNS, diagnostics

            da, db = diagnostics(p, st), diagnostics(p, ref)
            ty = COLUMNS.index("tip_y")
            rows[seed] = {"kind": "beam", "particles": int(p.solid_number),
                          "tip_y_error_m": abs(da[ty] - db[ty]), "tip_y_fp64_m": float(db[ty])}
    record("fp64_sweep_subset", {"case": "sweep scenes " + ", ".join(map(str, SWEEP_SUBSET)), "steps": steps,
                                 "form": "mixed, batched", "summary": rows})
    print(rows)
    for seed, r in rows.items():
        if r["kind"] == "dam_break":
            assert r["front"] < 5e-3 and r["mass"] < 1e-4, (seed, r)
        else:
            assert r["tip_y_error_m"] <= 5e-3 * max(abs(r["tip_y_fp64_m"]), 1e-6), (seed, r)
