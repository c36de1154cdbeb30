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


class Clocks:
    """nvidia-smi SM clock and throttle reasons sampled every 200 ms while
    the harness runs (the samples under load: SM clock above 1 GHz or power
    above 300 W)."""
    Q = ("clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.hw_slowdown,"
         "clocks_event_reasons.hw_thermal_slowdown,clocks_event_reasons.sw_thermal_slowdown,"
         "clocks_event_reasons.sw_power_cap")

    def __enter__(self):
        import subprocess
        import threading

        self.rows = []
        try:
            self.proc = subprocess.Popen(["nvidia-smi", "--id=0", f"--query-gpu={self.Q}",
                                          "--format=csv,noheader,nounits", "-lms", "200"],
                                         stdout=subprocess.PIPE, stderr=subprocess.DEVNULL, text=True)
        except OSError:
            self.proc = None
            return self

        def read():
            for line in self.proc.stdout:
                self.rows.append([c.strip() for c in line.split(",")])

        self.t = threading.Thread(target=read, daemon=True)
        self.t.start()
        return self

    def __exit__(self, *exc):
        if self.proc:
            self.proc.terminate()
            self.proc.wait(timeout=5)

    def summary(self) -> dict:
        import statistics

        def num(x):
            try:
                return float(x)
            except ValueError:
                return None

        rows = [r for r in self.rows if len(r) >= 7 and num(r[0]) is not None]
        load = [r for r in rows if num(r[0]) > 1000 or (num(r[2]) or 0) > 300]
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        reasons = sorted({names[k] for r in load for k in range(4) if r[3 + k].lower().startswith("active")})
        return {"samples": len(rows), "samples_under_load": len(load),
                "sm_mhz_median": statistics.median(num(r[0]) for r in load) if load else None,
                "sm_max_mhz": max(num(r[1]) for r in rows) if rows else None, "reasons": reasons}


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
        with Clocks() as clk:
            r = build_ref.run(cdir, ["time", str(a.warmup), str(a.steps)], run_dir=Path(t) / "run")
    if r.returncode:
        print(json.dumps({"case": a.case, "error": r.stderr[-500:]}))
        return 1
    res = json.loads(r.stdout.strip().splitlines()[-1])
    n = res["n_fluid"] + res["n_solid"]
    res.update(case=a.case, args=kw, particle_steps_per_s=n * 1e3 / res["ms_per_step"],
               impl="reference CUDA build (sm_103a, -use_fast_math, Eigen-subset shim)", clocks=clk.summary())
    print(json.dumps(res))
    return 0


if __name__ == "__main__":
    sys.exit(main())
