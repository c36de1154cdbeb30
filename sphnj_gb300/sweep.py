"""Steps the scene sweep (cases.sweep_scene) as one batch and prints the time.

    python -m sphnj_gb300.sweep [--scenes N] [--form mixed|plain] [--warmup W] [--steps K]
                                [--tile-h H | --autotune]

Scenes 0..N-1 of the sweep are created in the chosen form and stepped
together through sphnj_batch_step: W untimed steps, then K steps timed with
CUDA events on the batch's stream.  --tile-h sets the cells per tile of
the neighbour sweeps (16 by default); --autotune lets the batch's tuner
choose the sweep configuration first and prints its choice.  It is the batched leg of `bench.py`'s
sweep on its own, small enough to run under a profiler.
"""
from __future__ import annotations

import argparse

from . import Batch, Simulation, abi, cases


def main(argv=None) -> None:
    ap = argparse.ArgumentParser(prog="python -m sphnj_gb300.sweep")
    ap.add_argument("--scenes", type=int, default=cases.SWEEP_SCENES)
    ap.add_argument("--form", choices=["mixed", "plain"], default="mixed")
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--steps", type=int, default=2)
    ap.add_argument("--tile-h", type=int, default=16)
    ap.add_argument("--autotune", action="store_true")
    args = ap.parse_args(argv)
    import torch

    form = abi.FORM_MIXED if args.form == "mixed" else abi.FORM_PLAIN
    sims = []
    units = 0
    for s in range(args.scenes):
        case = cases.sweep_scene(s)
        p = case.params()
        units += p.fluid_number_total + p.solid_number
        sim = Simulation(p, form)
        sim.upload(case.arrays())
        sims.append(sim)
    stream = torch.cuda.Stream()
    with Batch(sims) as b:
        b.set_stream(stream.cuda_stream)
        b.set_tiling(True, args.tile_h)
        if args.autotune:
            print("autotune:", b.autotune())
        b.step(args.warmup)
        b.synchronize()
        e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        e0.record(stream)
        b.step(args.steps)
        e1.record(stream)
        b.synchronize()
        ms = e0.elapsed_time(e1) / max(args.steps, 1)
    for sim in sims:
        sim.close()
    print(f"{args.scenes} scenes, {units} particles, {args.form} form: {ms:.3f} ms/step, "
          f"{units / (ms / 1e3) / 1e6:.1f} M particle-steps/s")


if __name__ == "__main__":
    main()
