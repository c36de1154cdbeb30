"""Generates the golden fixtures in tests/golden/ from the SPHNJ reference's
own CUDA build (needs a GPU; the reference harness is built by
oracle/ref/build_ref.py from the reference sources).

For every case in FIXTURES: the case is generated with sphnj_gb300.cases,
written in the reference's case format, run through the reference harness
for `steps` steps, and the state dumps at the listed steps plus the global
diagnostics are stored as <name>.npz:
    s<step>/<field>   per-particle arrays and cell lists of the reference
    diag              rows: step front mom_x mom_y ek rho_sum tip_x tip_y eks eps
    maxspeed          rows: step max_speed (getMaxSpeed value of that step)
    ini               the input.ini text the reference read

    python tests/golden/make_fixtures.py [out_dir] [name ...]
"""
from __future__ import annotations

import json
import struct
import sys
import tempfile
from pathlib import Path

import numpy as np

ROOT = Path(__file__).resolve().parents[2]
sys.path.insert(0, str(ROOT))

from sphnj_gb300 import cases  # noqa: E402

# name -> (generator, kwargs, steps, dump steps, diag_every)
FIXTURES = {
    "water": ("dam_break_water", dict(dx=0.02, iend=2000), 2000, [0, 1, 51, 52, 199, 200], 10),
    "gas": ("dam_break_gas", dict(dx=0.05, iend=200), 200, [0, 1, 51, 52], 10),
    "beam": ("beam", dict(dx=0.002, iend=2000, cfl=0.25), 2000, [0, 1, 51, 52], 10),
    "gate": ("gate", dict(dx=0.002, gas=False, layers=3, substeps=4, iend=200), 200, [0, 1, 51, 52], 10),
    # the hydroelastic gate with air at 1000:1 (gas-liquid-solid coupling:
    # fluidSolidCalculate with gas fluid, solidFluidCouple from gas)
    "gate_air": ("gate", dict(dx=0.002, gas=True, layers=3, substeps=4, iend=200), 200, [0, 1, 51, 52], 10),
    "auxetic": ("auxetic_block", dict(dx=0.002, n=20, iend=200), 200, [0, 1, 51, 52, 200], 5),
}


# output fixtures: the reference's own Output functions run by the harness's
# `run` mode (DeviceCalculation::calculation with outputs); every file it
# writes under ..\\..\\out is stored as text under its path below out/.
# name -> (generator, kwargs, global writers)
OUTPUT_FIXTURES = {
    "out_water": ("dam_break_water", dict(dx=0.02, iend=100, extra_ini=dict(result_interval=50)),
                  "default,edge,total_energy"),
    # domain_xmax = beam length: outputEndPosition's point (xmax - d/2,
    # (ymin + ymax)/2 - d/2) is then the beam's end particle
    "out_beam": ("beam", dict(dx=0.002, cfl=0.25, iend=100, extra_ini=dict(result_interval=50, domain_xmax=0.2)),
                 "default,total_energy,end_position,crush_force"),
}


def make_case(name: str):
    gen, kw, *_ = FIXTURES[name]
    return cases.by_name(gen, **kw)


def read_dump(path: Path) -> tuple[int, dict]:
    b = path.read_bytes()
    assert b[:8] == b"SPHREF01", path
    step, n = struct.unpack_from("<ii", b, 8)
    off = 16
    out = {}
    for _ in range(n):
        name = b[off:off + 48].split(b"\0")[0].decode()
        dt = b[off + 48:off + 56].split(b"\0")[0].decode()
        (cnt,) = struct.unpack_from("<q", b, off + 56)
        off += 64
        dtype = {"f4": np.float32, "f8": np.float64, "i4": np.int32}[dt]
        nbytes = cnt * np.dtype(dtype).itemsize
        out[name] = np.frombuffer(b, dtype=dtype, count=cnt, offset=off).copy()
        off += nbytes
    return step, out


def run_case(name: str, out_dir: Path, work: Path) -> Path:
    sys.path.insert(0, str(ROOT / "oracle" / "ref"))
    import build_ref  # noqa: E402

    gen, kw, steps, dumps, diag_every = FIXTURES[name]
    case = make_case(name)
    cdir = case.write(work / name)
    prefix = (work / f"{name}_dump").resolve()
    r = build_ref.run(cdir, ["dump", str(steps), ",".join(map(str, dumps)), str(prefix), str(diag_every)],
                      run_dir=work / f"{name}_run")
    if r.returncode:
        raise RuntimeError(f"{name}: reference harness failed ({r.returncode})\n{r.stdout[-2000:]}\n{r.stderr[-2000:]}")
    arrays = {"ini": np.array(case.ini_text()), "generator": np.array(json.dumps([gen, kw]))}
    for s in dumps:
        step, d = read_dump(Path(f"{prefix}_{s:06d}.bin"))
        for k, v in d.items():
            arrays[f"s{s}/{k}"] = v
    arrays["diag"] = np.loadtxt(f"{prefix}_diag.txt", ndmin=2)
    ms = Path(f"{prefix}_maxspeed.txt")
    if ms.exists() and ms.stat().st_size:
        arrays["maxspeed"] = np.loadtxt(ms, ndmin=2)
    out = out_dir / f"{name}.npz"
    np.savez_compressed(out, **arrays)
    return out


def run_outputs(name: str, out_dir: Path, work: Path) -> Path:
    sys.path.insert(0, str(ROOT / "oracle" / "ref"))
    import build_ref  # noqa: E402

    gen, kw, globals_ = OUTPUT_FIXTURES[name]
    case = cases.by_name(gen, **kw)
    cdir = case.write(work / name)
    run_dir = work / f"{name}_run"
    r = build_ref.run(cdir, ["run", globals_], run_dir=run_dir)
    if r.returncode:
        raise RuntimeError(f"{name}: reference harness failed ({r.returncode})\n{r.stdout[-2000:]}\n{r.stderr[-2000:]}")
    prefix = "..\\..\\out\\"
    arrays = {"ini": np.array(case.ini_text()), "generator": np.array(json.dumps([gen, kw])),
              "globals": np.array(globals_)}
    for f in sorted(run_dir.iterdir()):
        if f.is_file() and f.name.startswith(prefix):
            arrays["out/" + f.name[len(prefix):].replace("\\", "/")] = np.array(f.read_text())
    out = out_dir / f"{name}.npz"
    np.savez_compressed(out, **arrays)
    return out


def main(argv):
    out_dir = Path(argv[1]) if len(argv) > 1 else Path(__file__).resolve().parent
    names = argv[2:] or list(FIXTURES) + list(OUTPUT_FIXTURES)
    out_dir.mkdir(parents=True, exist_ok=True)
    sys.path.insert(0, str(ROOT / "oracle" / "ref"))
    import build_ref  # noqa: E402

    build_ref.build()
    with tempfile.TemporaryDirectory() as t:
        for n in names:
            p = (run_outputs if n in OUTPUT_FIXTURES else run_case)(n, out_dir, Path(t))
            print(n, p, p.stat().st_size, flush=True)


if __name__ == "__main__":
    main(sys.argv)
