"""Times the SPHNJ reference's own CUDA build on a generated case - test
infrastructure (the reference's GPU throughput beside this library's).

The case is written in the reference's format; the harness (build_ref.py)
runs `warmup` steps, then `steps` timed steps of the reference's own stage
functions (calculation.cu:32-42 without the output calls), including the
per-step device-to-host copy of every fluid velocity that getMaxSpeed does
(fluid.cu:429-440) and the cudaDeviceSynchronize after every launch.

    python oracle/ref/time_reference.py <case> [key=value ...] [--warmup W] [--steps K]
    e.g.  python oracle/ref/time_reference.py dam_break_gas dx=0.0017 --steps 10
"""
from __future__ import annotations

import argparse
import json
import sys
import tempfile
from pathlib import Path

HERE = Path(__file__).resolve().parent
sys.path.insert(0, str(HERE.parents[1]))
sys.path.insert(0, str(HERE))

import build_ref  # noqa: E402
from sphnj_gb300 import cases  # noqa: E402


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("case")
    ap.add_argument("kw", nargs="*")
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--steps", type=int, default=10)
    a = ap.parse_args()
    kw = {}
    for item in a.kw:
        k, v = item.split("=", 1)
        kw[k] = float(v) if any(ch in v for ch in ".e") else int(v)
    case = cases.by_name(a.case, **kw)
    build_ref.build()
    with tempfile.TemporaryDirectory() as t:
        cdir = case.write(Path(t) / "case")
        r = build_ref.run(cdir, ["time", str(a.warmup), str(a.steps)], run_dir=Path(t) / "run")
    if r.returncode:
        print(json.dumps({"case": a.case, "error": r.stderr[-500:]}))
        return 1
    res = json.loads(r.stdout.strip().splitlines()[-1])
    n = res["n_fluid"] + res["n_solid"]
    res.update(case=a.case, args=kw, particle_steps_per_s=n * 1e3 / res["ms_per_step"],
               impl="reference CUDA build (sm_103a, -use_fast_math, Eigen-subset shim)")
    print(json.dumps(res))
    return 0


if __name__ == "__main__":
    sys.exit(main())
