#!/usr/bin/env python
"""Throughput of SPHNJ's particle-step hot path on GB300 (particle-steps/s).

Workload (default): the 4.15M-particle gas-liquid dam break - 1.0 x 2.0 m
water column in a 4.0 x 3.0 m tank filled with air (rho 1.0), dx = 0.0017,
h = 1.2 dx, 3 wall layers (~24.7k virtual particles), 10 shifting passes per
step; synthetic lattice input generated by sphnj_gb300.cases.  One step = one
fluid step (cell ids, lists, virtual particles, pair pass, update, max speed,
10 shifting passes).  particle-steps/s = (N_fluid + N_solid) x steps / s.
The headline is the mixed-precision form (--form plain: the reference's
precision); the other form is timed beside it ("forms"), and the 256-scene
sweep is run scene by scene in the plain form and batched in both forms
("batched_sweep").

  python bench.py [--gpus N] [--steps K] [--warmup W] [--impl ours|reference]

N > 1 (torchrun): every rank runs its own replica of the scene (the path has
no data-path collective: scenes are independent), value = all ranks'
particle-steps / max time over ranks ("scaling": "weak").
--impl reference times the reference's CPU restatement (the oracle port: the
reference itself has only a CUDA implementation) on the host cores.
"""
from __future__ import annotations

import argparse
import json
import os
import statistics
import subprocess
import sys
import threading
import time
from pathlib import Path

import numpy as np

ROOT = Path(__file__).resolve().parent
sys.path.insert(0, str(ROOT))

METRIC = "particle-steps/s (1 GB300): mixed-prec+batched vs plain at stated FP64 error"
UNIT = "particle-steps/s"


def parse():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=50)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", default="ours", choices=["ours", "reference"])
    ap.add_argument("--dx", type=float, default=0.0017)
    ap.add_argument("--cpu-steps", type=int, default=10,
                    help="timed oracle steps of the CPU baseline on the workload (~10 s on 16 host cores)")
    ap.add_argument("--no-cpu-baseline", action="store_true")
    ap.add_argument("--no-e2e", action="store_true")
    ap.add_argument("--untiled", action="store_true", help="one thread per particle in the neighbour sweeps")
    ap.add_argument("--tile-h", type=int, default=16, help="cells per tile of the neighbour sweeps")
    ap.add_argument("--no-graphs", action="store_true", help="issue every kernel of a step instead of replaying "
                                                             "the step's captured CUDA graph")
    ap.add_argument("--form", default="mixed", choices=["plain", "mixed"],
                    help="form of the headline (the other is timed beside it): mixed, the mixed-precision "
                         "form the metric names (default), or plain, the reference's precision")
    ap.add_argument("--no-sweep", action="store_true", help="skip the 256-scene batched sweep")
    ap.add_argument("--sweep-steps", type=int, default=20, help="timed steps of the 256-scene sweep")
    ap.add_argument("--no-autotune", action="store_true",
                    help="batched sweep: keep --tile-h and the default block sizes instead of autotuning")
    return ap.parse_args()


def dist_env():
    return (int(os.environ.get("RANK", 0)), int(os.environ.get("WORLD_SIZE", 1)),
            int(os.environ.get("LOCAL_RANK", 0)))


class ClockSampler:
    """nvidia-smi clocks and throttle reasons sampled during the timed region."""
    Q = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,clocks_event_reasons.hw_slowdown,"
         "clocks_event_reasons.hw_thermal_slowdown,clocks_event_reasons.sw_thermal_slowdown,"
         "clocks_event_reasons.sw_power_cap")

    def __init__(self, gpu_index: int):
        self.idx = gpu_index
        self.rows = []
        self.proc = None

    def __enter__(self):
        try:
            self.proc = subprocess.Popen(["nvidia-smi", f"--id={self.idx}", f"--query-gpu={self.Q}",
                                          "--format=csv,noheader,nounits", "-lms", "100"],
                                         stdout=subprocess.PIPE, stderr=subprocess.DEVNULL, text=True)
            self.t = threading.Thread(target=self._read, daemon=True)
            self.t.start()
        except (FileNotFoundError, OSError):
            self.proc = None
        return self

    def _read(self):
        for line in self.proc.stdout:
            self.rows.append([c.strip() for c in line.split(",")])

    def __exit__(self, *a):
        if self.proc:
            self.proc.terminate()
            try:
                self.proc.wait(timeout=5)
            except subprocess.TimeoutExpired:
                self.proc.kill()

    def summary(self):
        sm = [float(r[1]) for r in self.rows if len(r) >= 9 and r[1].replace(".", "").isdigit()]
        mx = [float(r[2]) for r in self.rows if len(r) >= 9 and r[2].replace(".", "").isdigit()]
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        reasons = sorted({names[k] for r in self.rows if len(r) >= 9 for k in range(4)
                          if r[5 + k].lower().startswith("active")})
        return {"sm_mhz": statistics.median(sm) if sm else None, "sm_max_mhz": max(mx) if mx else None,
                "reasons": reasons, "samples": len(sm)}


def make_case(dx):
    from sphnj_gb300 import cases

    return cases.dam_break_gas(dx=dx)


def cpu_model() -> str:
    """The host CPU's model name (x86 'model name', or lscpu's 'Model name'
    on Arm, where /proc/cpuinfo lists only part numbers)."""
    try:
        for line in Path("/proc/cpuinfo").read_text().splitlines():
            if line.lower().startswith("model name"):
                return line.split(":", 1)[1].strip()
    except OSError:
        pass
    try:
        out = subprocess.run(["lscpu"], capture_output=True, text=True, timeout=10).stdout
        for line in out.splitlines():
            if line.strip().lower().startswith("model name"):
                return line.split(":", 1)[1].strip()
    except (OSError, subprocess.SubprocessError):
        pass
    return "unknown"


def next_sort_step(step: int, every: int) -> int:
    """Steps to take from step counter `step` so that the next step taken is
    a sort step ((i - 1) mod sort_every_step == 0, SimTime::isSort)."""
    return (-step) % every


def oracle_sim(case, threads=0):
    """The oracle (reference precision) uploaded with the case; its
    parameters derived by the oracle itself, so that the product library is
    never loaded on this path."""
    import oracle

    p = oracle.params_for(case)
    if threads:
        oracle.set_threads(threads)
    o = oracle.OracleSim(p, oracle.REFERENCE_PRECISION, threads=threads)
    o.upload(case.arrays())
    return o, p


def oracle_timed(o, p, warm, steps, align):
    """Times `steps` oracle steps after `warm` untimed ones; with `align` the
    step counter is moved on (untimed, no work) so that the timed steps start
    with a sort step, as the GPU arm's do.  Returns seconds."""
    import oracle  # noqa: F401

    o.step(warm)
    if align:
        o.set_step(o.step_index + next_sort_step(o.step_index, p.sort_every_step))
    t0 = time.perf_counter()
    o.step(steps)
    return time.perf_counter() - t0


RECORDS = ROOT / "tests" / "records"


def error_records() -> dict:
    """The errors against the FP64 oracle that the GPU tests measured and
    recorded (tests/records/*.json, written by tests/test_gpu_fp64_error.py
    with SPHNJ_RECORD_DIR set): per record, its case and the largest errors of
    each form."""
    out = {}
    for f in sorted(RECORDS.glob("fp64_*.json")):
        try:
            rec = json.loads(f.read_text())
        except (OSError, ValueError):
            continue
        out[f.stem] = rec.get("summary", rec)
    return out or {"missing": "no error records under tests/records"}


def run_reference(args):
    """The reference's CPU implementation of the path on this host: the
    reference has only a CUDA implementation, so this is its CPU restatement
    (the oracle port, OpenMP over particles) on the same workload as the GPU
    arm - the 4.15M-particle dam break - with every host thread; W warm-up
    steps, then K timed steps that start with a sort step.  A 1-thread step
    is timed beside it."""
    rank, world, _ = dist_env()
    if rank != 0:
        return 0
    import oracle

    oracle.build()
    case = make_case(args.dx)
    t0 = time.perf_counter()
    o, p = oracle_sim(case)
    setup = time.perf_counter() - t0
    n = p.fluid_number_total + p.solid_number
    threads = oracle.max_threads()
    dt = oracle_timed(o, p, max(args.warmup, 1), args.steps, align=True)
    v = n * args.steps / dt
    oracle.set_threads(1)
    t1 = time.perf_counter()
    o.step(1)
    dt1 = time.perf_counter() - t1
    oracle.set_threads(threads)
    o.close()
    sample = (f"the full workload ({n} particles), {args.warmup} warm-up steps, then {args.steps} timed steps "
              f"starting with a sort step, {threads} threads; 1 thread: {n / dt1:.4g} particle-steps/s over one "
              f"step")
    line = {
        "impl": "reference", "metric": METRIC, "value": v, "unit": UNIT, "n_gpus": args.gpus,
        "steps": args.steps, "warmup": args.warmup, "ms_per_step": dt * 1e3 / args.steps,
        "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f32",
        "data": "synthetic (lattice dam break generated in-process)",
        "config": {"workload": f"gas-liquid dam break, 1.0x2.0 m water in a 4.0x3.0 m air-filled tank, dx={args.dx}",
                   "particles": n, "n_fluid": p.fluid_number_total, "n_virt": p.virt_number,
                   "shift_per_step": p.shift_per_step, "sort_every_step": p.sort_every_step},
        "cpu_baseline": {"value": v, "unit": UNIT, "cores": threads, "kind": "port", "sample": sample,
                         "one_thread": n / dt1, "cpu": cpu_model(), "setup_s": setup},
        "e2e": {"value": v, "unit": UNIT, "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0},
        "note": "the reference has no CPU implementation of the path (CUDA only); this arm is its CPU "
                "restatement in oracle/ (OpenMP), with parameters derived by the oracle itself",
    }
    print(json.dumps(line), flush=True)
    return 0


def run_sweep(args, stream, peak):
    """The 256-scene sweep (sphnj_gb300.cases.sweep_scene, seeds 0..255: 128
    water dam breaks of 2k-60k particles, 128 beams of 1k-20k): the plain
    form run scene by scene (each scene's steps as its own graph launches, the
    scenes one after another on one stream), then the same scenes advanced as
    one batch (one launch per stage over all scenes).  Both timed with CUDA
    events on that stream after `warmup` steps; the state (~0.4 GB) exceeds L2."""
    import torch

    import sphnj_gb300 as S
    from sphnj_gb300 import abi, byte_model, cases

    from sphnj_gb300.sharding import balanced_partition

    rank, world, _ = dist_env()
    t0 = time.perf_counter()
    scenes = [cases.sweep_scene(s) for s in range(cases.SWEEP_SCENES)]
    all_params = [c.params() for c in scenes]
    weights = [p.fluid_number_total + p.solid_number for p in all_params]
    # one process per GPU: this rank's particle-balanced share of the scenes
    mine = balanced_partition(weights, world)[rank]
    params = [all_params[i] for i in mine]
    arrays = [scenes[i].arrays() for i in mine]
    setup_s = time.perf_counter() - t0
    units = sum(weights)  # all ranks' particles: the whole-job rate
    K = args.sweep_steps

    def timed(fn):
        if world > 1:
            torch.distributed.barrier()
        torch.cuda.synchronize()
        e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        e0.record(stream)
        fn()
        e1.record(stream)
        torch.cuda.synchronize()
        ms = e0.elapsed_time(e1)
        if world > 1:
            t = torch.tensor([ms], device="cuda")
            torch.distributed.all_reduce(t, op=torch.distributed.ReduceOp.MAX)
            ms = float(t.item())
        return ms

    def make(form):
        sims = []
        for p, a in zip(params, arrays):
            sim = S.Simulation(p, form)
            sim.set_stream(stream.cuda_stream)
            sim.set_tiling(True, args.tile_h)
            sim.upload(a)
            sims.append(sim)
        return sims

    def rate(ms):
        return {"value": units * K / (ms / 1e3), "ms_per_step": ms / K}

    # plain form, scene by scene
    sims = make(abi.FORM_PLAIN)
    for sim in sims:
        sim.step(args.warmup)
    lp0 = sum(sim.launches() for sim in sims)
    ms_plain = timed(lambda: [sim.step(K) for sim in sims])
    launches_plain = sum(sim.launches() for sim in sims) - lp0
    for sim in sims:
        sim.synchronize()
        sim.close()

    # batched, each form
    out = {}
    for name, form in (("batched", abi.FORM_PLAIN), ("batched_mixed", abi.FORM_MIXED)):
        sims = make(form)
        b = S.Batch(sims)
        b.set_stream(stream.cuda_stream)
        b.set_tiling(True, args.tile_h)
        # the launch shape and each size class's tile height chosen by the
        # library's autotuner on the first step's state (the state is put
        # back), then the warm-up steps, which capture the chosen shape's graphs
        b.step(1)
        tuned = None if args.no_autotune else b.autotune(steps=3)
        b.step(args.warmup)
        l0 = b.launches()
        ms = timed(lambda: b.step(K))
        launches = b.launches() - l0
        b.synchronize()
        b.profile_enable(True)
        b.step(K)
        prof = b.profile_read()
        b.profile_enable(False)
        b.close()
        for sim in sims:
            sim.close()
        total = sum(v[0] for v in prof.values())
        mixed = form == abi.FORM_MIXED
        sweep_bytes = sum(byte_model.step_bytes(q.fluid_number_total, q.solid_number, q.virt_number,
                                                q.shift_per_step, q.solid_sub_step, mixed) for q in params)
        achieved = sweep_bytes / (ms / K / 1e3) / 1e9
        out[name] = dict(rate(ms), launches_per_step=launches / K, autotuned=tuned,
                         roofline={"bound": "hbm", "what": "whole batched step: compulsory bytes of every scene's "
                                                           "passes (byte model) / step time",
                                   "bytes_per_step": sweep_bytes, "achieved": achieved, "peak": peak,
                                   "unit": "GB/s", "frac": achieved / peak},
                         stage_share={k: round(v[0] / total, 4) for k, v in prof.items() if v[1]})
        out[name + "_over_plain"] = ms_plain / ms
    return {
        "workload": "256 independent scenes (seeds 0..255): 128 water dam breaks of 2k-60k particles "
                    "(H/W in [0.5, 2.5]), 128 cantilever beams of 1k-20k particles (E 0.5-20 MPa, "
                    "nu 0.3-0.45, L 0.1-0.3 m), +-0.01 dx jitter",
        "scenes": len(all_params), "particles": units, "steps": K, "warmup": args.warmup,
        "sharding": f"{world} rank(s), particle-balanced scene partition, no data-path collective",
        "plain_scene_by_scene": dict(rate(ms_plain), launches_per_step=launches_plain / K),
        **out,
        "setup_s": setup_s,
        "forms": "plain: reference precision; mixed: FP32 pair loops, cell + offset positions with Kahan "
                 "integration, FP64 correction inverse and F/PK1 step",
    }


def run_ours(args):
    import torch

    import sphnj_gb300 as S
    from sphnj_gb300 import abi, byte_model

    rank, world, local = dist_env()
    torch.cuda.set_device(local)
    if world > 1:
        import torch.distributed as dist

        dist.init_process_group("nccl", device_id=torch.device("cuda", local))
    S.build()
    case = make_case(args.dx)
    p = case.params()
    arr = case.arrays()
    nf, ns, nv = p.fluid_number_total, p.solid_number, p.virt_number
    units = nf + ns
    stream = torch.cuda.Stream()
    form = abi.FORM_MIXED if args.form == "mixed" else abi.FORM_PLAIN
    sim = S.Simulation(p, form)
    sim.set_stream(stream.cuda_stream)
    sim.set_tiling(not args.untiled, args.tile_h)
    sim.set_graphs(not args.no_graphs)
    sim.upload(arr)
    # launch shape chosen by the library's autotuner on the first step's state
    # (tile height, lists, block sizes; the state is put back)
    tuned = None
    if not args.no_autotune and not args.untiled:
        sim.step(1)
        tuned = sim.autotune(steps=3)

    def barrier():
        if world > 1:
            torch.distributed.barrier()

    # warm-up, then on to the step before a sort step, so that the timed
    # steps start with a sort (sort_every_step = 50: one sort in K = 20 timed
    # steps over-weights it; the amortised rate over one whole sort period is
    # measured below as "sort_period").  The warm-up runs through one sort
    # step first, so that the graph of every kind of step the timed region
    # meets is captured before it.
    sim.step(args.warmup)
    sim.step(next_sort_step(sim.step_index, p.sort_every_step) + 1)
    sim.step(next_sort_step(sim.step_index, p.sort_every_step))
    sim.synchronize()
    first_timed = sim.step_index + 1

    # ---- timed region: inputs resident in HBM (state 0.3 GB > 129 MB L2) ---
    l0 = sim.launches()
    with ClockSampler(torch.cuda.current_device()) as clk:
        barrier()
        torch.cuda.synchronize()
        e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        e0.record(stream)
        sim.step(args.steps)
        e1.record(stream)
        torch.cuda.synchronize()
        barrier()
    launches = sim.launches() - l0
    sim.synchronize()
    ms = e0.elapsed_time(e1)
    if world > 1:
        t = torch.tensor([ms], device="cuda")
        torch.distributed.all_reduce(t, op=torch.distributed.ReduceOp.MAX)
        ms = float(t.item())
    value = units * world * args.steps / (ms / 1e3)

    # ---- one whole sort period (sort_every_step steps from a sort step) ------
    sim.step(next_sort_step(sim.step_index, p.sort_every_step))
    sim.synchronize()
    q0, q1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    q0.record(stream)
    sim.step(p.sort_every_step)
    q1.record(stream)
    torch.cuda.synchronize()
    ms_period = q0.elapsed_time(q1)
    sort_period = {"steps": p.sort_every_step, "ms_per_step": ms_period / p.sort_every_step,
                   "value": units * world * p.sort_every_step / (ms_period / 1e3),
                   "what": "one sort step and the incremental steps up to the next sort, timed together"}

    # ---- per-stage device times (CUDA events on the launching stream) -------
    sim.profile_enable(True)
    sim.step(args.steps)
    prof = sim.profile_read()
    sim.profile_enable(False)
    total_ms = sum(v[0] for v in prof.values())
    dom = max(prof, key=lambda k: prof[k][0])
    d_ms, d_calls, d_kern = prof[dom]
    avg_ms = d_ms / max(d_calls, 1)
    mixed = form == abi.FORM_MIXED
    bpl = byte_model.bytes_per_launch(dom, nf, ns, nv, mixed, shifts=p.shift_per_step)
    peaks = {}
    try:
        peaks = json.loads((ROOT / "MEASURED_PEAKS.json").read_text())
    except (OSError, ValueError):
        pass
    peak = float(peaks.get("hbm_gbs", 6800.0))
    achieved = bpl / (avg_ms / 1e3) / 1e9
    roofline = {"bound": "hbm", "kernel": dom, "achieved": achieved, "peak": peak, "unit": "GB/s",
                "frac": achieved / peak,
                "traffic": byte_model.measured_traffic_per_launch(dom, nf, mixed) if args.tile_h == 16 and not args.untiled
                else None,
                "traffic_source": "ncu dram bytes of one launch at 2.08M particles, scaled by particle count "
                                  "(captured before the particles next to a wall got neighbour lists)",
                "peak_source": "MEASURED_PEAKS.json hbm_gbs (measured)" if peaks else "fallback 6.8 TB/s",
                "bytes_per_launch": bpl, "avg_launch_ms": avg_ms,
                # the DRAM bytes ncu measured for such a launch over the same
                # CUDA-event time: the rate the kernel actually draws
                "dram_gbs": (byte_model.measured_traffic_per_launch(dom, nf, mixed) / (avg_ms / 1e3) / 1e9
                             if byte_model.measured_traffic_per_launch(dom, nf, mixed) and args.tile_h == 16
                             and not args.untiled else None),
                "issue_slots_busy": dict(byte_model.ISSUE_ACTIVE_MIXED if mixed else byte_model.ISSUE_ACTIVE,
                                         source="ncu smsp__issue_active of one launch at 2.08M particles"),
                "stage_share": {k: round(v[0] / total_ms, 4) for k, v in prof.items() if v[1]}}
    step_bytes = byte_model.step_bytes(nf, ns, nv, p.shift_per_step, p.solid_sub_step, mixed)

    # ---- end to end through the C ABI with pinned host buffers ---------------
    e2e = None
    if not args.no_e2e:
        mask = abi.F_FLUID_KINEMATICS | abi.F_FLUID_THERMO

        # the library's pinned, device-mapped host memory: each transfer is
        # one kernel reading or writing the host arrays over the host link
        io_fields = ("fluid_position", "fluid_velocity", "fluid_density", "fluid_pressure")
        hin = sim.host_state(io_fields)
        hout = sim.host_state(io_fields)
        sim.download(mask, into=hin)  # start from the current state
        h2d = sum(a.nbytes for a in hin.values())
        d2h = sum(a.nbytes for a in hout.values())
        ke = max(5, args.steps // 2)

        def timed_loop(one_step):
            nonlocal hin, hout
            barrier()
            torch.cuda.synchronize()
            t0 = time.perf_counter()
            for _ in range(ke):
                one_step(hin, hout)
                hin, hout = hout, hin
            torch.cuda.synchronize()
            dt = time.perf_counter() - t0
            if world > 1:
                t = torch.tensor([dt], device="cuda")
                torch.distributed.all_reduce(t, op=torch.distributed.ReduceOp.MAX)
                dt = float(t.item())
            return dt

        # three calls per step, each part timed on the host
        part = [0.0, 0.0, 0.0]  # upload (returns when copied), step (enqueue), download (waits for the step)

        def three_calls(a, b):
            ta = time.perf_counter()
            sim.upload_fields(mask, a)
            tb = time.perf_counter()
            sim.step(1)
            tc = time.perf_counter()
            sim.download(mask, into=b)
            td = time.perf_counter()
            part[0] += tb - ta
            part[1] += tc - tb
            part[2] += td - tc

        dt3 = timed_loop(three_calls)
        # one call per step: the same transfers overlapped with the step
        dt1 = timed_loop(lambda a, b: sim.step_exchange(1, mask, a, mask, b))
        e2e = {"value": units * world * ke / dt1, "unit": UNIT, "h2d_bytes_per_step": h2d, "d2h_bytes_per_step": d2h,
               "steps": ke, "api": "sphnj_step_exchange(1): upload, step and download in one call per step",
               "host_memory": "sphnj_host_alloc (pinned, device-mapped)",
               "ms_per_step": dt1 * 1e3 / ke,
               "three_calls": {"value": units * world * ke / dt3, "ms_per_step": dt3 * 1e3 / ke,
                               "api": "sphnj_upload_fields + sphnj_step(1) + sphnj_download per step",
                               "ms_per_step_parts": {"upload": part[0] * 1e3 / ke, "step_enqueue": part[1] * 1e3 / ke,
                                                     "step_and_download": part[2] * 1e3 / ke}}}

    normals = sim.download(abi.F_VIRT)["virt_normal"].copy()
    sim.close()

    # the other form on the same workload, timed the same way
    other = abi.FORM_PLAIN if form == abi.FORM_MIXED else abi.FORM_MIXED
    with S.Simulation(p, other) as o:
        o.set_stream(stream.cuda_stream)
        o.set_tiling(not args.untiled, args.tile_h)
        o.set_graphs(not args.no_graphs)
        o.upload(arr)
        tuned_other = None
        if not args.no_autotune and not args.untiled:
            o.step(1)
            tuned_other = o.autotune(steps=3)
        o.step(args.warmup)
        # the same timed window as the headline's: starting with a sort step
        o.step(next_sort_step(o.step_index, p.sort_every_step) + 1)
        o.step(next_sort_step(o.step_index, p.sort_every_step))
        o.synchronize()
        barrier()
        torch.cuda.synchronize()
        f0, f1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        f0.record(stream)
        o.step(args.steps)
        f1.record(stream)
        torch.cuda.synchronize()
        o.synchronize()
        ms_other = f0.elapsed_time(f1)
    if world > 1:
        t = torch.tensor([ms_other], device="cuda")
        torch.distributed.all_reduce(t, op=torch.distributed.ReduceOp.MAX)
        ms_other = float(t.item())
    names = {abi.FORM_PLAIN: "plain", abi.FORM_MIXED: "mixed"}
    forms = {names[form]: {"value": value, "ms_per_step": ms / args.steps, "autotuned": tuned},
             names[other]: {"value": units * world * args.steps / (ms_other / 1e3),
                            "ms_per_step": ms_other / args.steps, "autotuned": tuned_other}}
    forms["mixed_over_plain"] = forms["plain"]["ms_per_step"] / forms["mixed"]["ms_per_step"]
    forms["error_vs_fp64_oracle"] = error_records()

    sweep = None
    if not args.no_sweep:
        sweep = run_sweep(args, stream, peak)

    cpu = None
    if rank == 0 and world == 1 and not args.no_cpu_baseline:
        import oracle

        o, cp = oracle_sim(case)
        cores = oracle.max_threads()
        dt = oracle_timed(o, cp, 1, args.cpu_steps, align=False)
        v = units * args.cpu_steps / dt
        oracle.set_threads(1)
        t1 = time.perf_counter()
        o.step(1)
        dt1 = time.perf_counter() - t1
        oracle.set_threads(cores)
        o.close()
        cpu = {"value": v, "unit": UNIT, "cores": cores, "kind": "port", "cpu": cpu_model(), "one_thread": units / dt1,
               "sample": f"oracle (reference precision, OpenMP) on this workload ({units} particles), one sort "
                         f"step untimed, then {args.cpu_steps} steps ({dt:.1f} s); one_thread: one more step on 1 "
                         f"thread ({dt1:.1f} s)"}

    if world > 1:
        torch.distributed.destroy_process_group()
    if rank != 0:
        return 0
    line = {
        "metric": METRIC, "value": value, "unit": UNIT, "n_gpus": world, "steps": args.steps,
        "warmup": args.warmup, "ms_per_step": ms / args.steps, "higher_is_better": True, "scaling": "weak",
        "vs_baseline": None, "dtype": "f32",
        "data": "synthetic (lattice gas-liquid dam break generated in-process, reference .dat layout)",
        "config": {"workload": f"gas-liquid dam break, 1.0x2.0 m water in a 4.0x3.0 m air-filled tank, dx={args.dx}",
                   "form": "plain (reference precision and cell-list order)" if form == abi.FORM_PLAIN else
                           "mixed (FP32 pair loops, cell + offset positions with Kahan integration)",
                   "sweeps": "per-particle" if args.untiled else
                             (f"tiled, {args.tile_h} cells per tile" if tuned is None else
                              f"tiled, autotuned: {tuned['tile_h']} cells per tile, lists {tuned['lists']}, "
                              f"blocks {tuned['shift_block'] or 'default'} (shifting) / "
                              f"{tuned['pair_block'] or 'default'} (pair)"),
                   "launch": "direct" if args.no_graphs else "one CUDA graph per kind of step", "n_fluid": nf, "n_liquid": p.fluid_number[0],
                   "n_solid": ns, "n_virt": nv, "cells": p.cell_number_total, "shift_per_step": p.shift_per_step,
                   "sort_every_step": p.sort_every_step, "dt": p.dt,
                   "l2": "inputs larger than L2 (fluid state ~0.3 GB > 129 MB)",
                   "parallelism": f"replicas x{world}" if world > 1 else "single GPU",
                   "byte_model_bytes_per_step": step_bytes,
                   "step_hbm_frac_of_byte_model": step_bytes / (ms / args.steps / 1e3) / 1e9 / peak},
        "roofline": roofline,
        "cpu_baseline": cpu,
        "e2e": e2e,
        "gpu_launches": launches,
        "timed_steps": f"{first_timed}..{first_timed + args.steps - 1} (starts with a sort step)",
        "sort_period": sort_period,
        "clocks": clk.summary(),
        "forms": forms,
        "batched_sweep": sweep,
    }
    print(json.dumps(line), flush=True)
    return 0


def relaunch_distributed(args) -> int:
    """bench.py --gpus N (N > 1) started without torchrun: runs itself as N
    processes under torch.distributed.run (one per GPU, rendezvous on
    127.0.0.1), as the multi-GPU launch does."""
    import socket

    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        port = s.getsockname()[1]
    cmd = [sys.executable, "-m", "torch.distributed.run", "--nnodes=1", f"--nproc-per-node={args.gpus}",
           "--master-addr", "127.0.0.1", f"--master-port={port}", str(ROOT / "bench.py"), *sys.argv[1:]]
    return subprocess.call(cmd)


def main():
    args = parse()
    if args.gpus > 1 and "WORLD_SIZE" not in os.environ:
        return relaunch_distributed(args)
    if args.impl == "reference":
        return run_reference(args)
    return run_ours(args)


if __name__ == "__main__":
    sys.exit(main())
