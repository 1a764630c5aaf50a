"""Autotuner for the batched ensemble step.

The knobs are the shapes the batched kernels take from nyxpm_tuning: the CIC
deposit tile (8x8x8, 8x8x4 or 16x8x4 cells per work item), the sort bucket (256,
512 or 1024 particles per work item of the counting sort and the kicks), the
number of plane rows per multigrid work item (the smoother block height), the
number of FP32 V-cycles per FP64 defect-correction iteration, and whether the
black-only prolongation covers four fine rows per task.  The tuner runs coordinate
descent on a scratch ensemble built from a size-stratified sample of the real
boxes: for each knob in turn it times a few steps per candidate value (CUDA
events inside nyxpm_ensemble_step, after a warm-up step that captures the new
graphs) with the other knobs at their best so far, every candidate from the
same ICs and a.  Results are cached in a
JSON file keyed by GPU name and the ensemble's size mix, so a serving process
tunes once per workload shape.
"""
from __future__ import annotations

import json
import os
import time

import numpy as np

from .ensemble import Ensemble, box_ics

CANDIDATES = {
    "deposit_tile": (0, 1, 2),
    "sort_bucket": (256, 512, 1024),
    "smooth_rows": (2, 4, 8),
    "inner_vcycles": (1, 2, 3),
    "prolong_quad": (1, 0),
}


def _gpu_name(ctx) -> str:
    try:
        import torch
        return torch.cuda.get_device_name(ctx.params.device)
    except Exception:
        return "cuda"


def signature(specs) -> str:
    mix = {}
    for s in specs:
        mix[s.n] = mix.get(s.n, 0) + 1
    return ",".join(f"{n}x{c}" for n, c in sorted(mix.items()))


def _sample(specs, max_boxes):
    by_n = {}
    for s in specs:
        by_n.setdefault(s.n, []).append(s)
    total = len(specs)
    out = []
    for n, group in sorted(by_n.items()):
        k = max(1, int(round(max_boxes * len(group) / total)))
        out.extend(group[:k])
    return out[:max(max_boxes, len(by_n))]


def tune(ctx, specs, a_start=0.02, da=0.009, steps=2, max_boxes=48, cache_path=None,
         ic_provider=None, verbose=False):
    """Return the best nyxpm_tuning values (dict) for this ensemble mix.
    ic_provider(spec) -> (pos, vel, mass) supplies the ICs of a sampled box
    (default: generate them)."""
    key = f"{_gpu_name(ctx)}|{signature(specs)}"
    cache = {}
    if cache_path and os.path.exists(cache_path):
        try:
            with open(cache_path) as f:
                cache = json.load(f)
        except Exception:
            cache = {}
    if key in cache:
        return dict(cache[key]["tuning"], cached=True)
    sample = _sample(specs, max_boxes)
    arena = int(sum(Ensemble.box_bytes(s.n, s.np) for s in sample) * 1.3) + (256 << 20)
    ens = Ensemble(ctx, arena)
    slots, ics = [], []
    for s in sample:
        if ic_provider is not None:
            pos, vel, mass = ic_provider(s)
        else:
            ic = box_ics(s, a_start)
            pos, vel, mass = ic.pos, ic.vel, ic.mass
        slot = ens.add(s.n, s.L, s.np)
        ens.upload(slot, pos, vel, mass)
        slots.append(slot)
        ics.append((pos, vel, mass))
    best = ens.tuning()
    a = [a_start]

    def restart():
        # every candidate starts from the same ICs at the same a: the solve's
        # cost changes with a, and a candidate timed later in the run would
        # otherwise be timed on a different state
        for slot, (pos, vel, mass) in zip(slots, ics):
            ens.upload(slot, pos, vel, mass)
        a[0] = a_start

    def run(n_steps):
        ms = 0.0
        for _ in range(n_steps):
            a0 = a[0]
            a1 = a0 + da
            win = 1.01 * da / min(a0 * ctx.hubble(a0), a1 * ctx.hubble(a1))
            dt = ctx.integrate_comoving_a_to_a(a0, a1, win)
            a1 = ctx.integrate_comoving_a(a0, dt)
            info = ens.step({s: a0 for s in slots}, {s: a1 for s in slots}, {s: dt for s in slots})
            ms += info["ms"]
            a[0] = a1
        return ms

    timings = {}
    t0 = time.time()
    for knob, values in CANDIDATES.items():
        res = {}
        for v in values:
            ens.set_tuning(**dict(best, **{knob: v}))
            restart()
            run(1)                      # the initial solve, graph capture, warm-up
            res[v] = run(steps) / steps
        timings[knob] = res
        best[knob] = min(res, key=res.get)
        if verbose:
            print(f"autotune {knob}: {res} -> {best[knob]}")
    ens.close()
    entry = {"tuning": best, "timings_ms_per_step": {k: {str(v): t for v, t in r.items()}
                                                     for k, r in timings.items()},
             "sample_boxes": len(sample), "seconds": time.time() - t0}
    if cache_path:
        cache[key] = entry
        os.makedirs(os.path.dirname(os.path.abspath(cache_path)), exist_ok=True)
        with open(cache_path, "w") as f:
            json.dump(cache, f, indent=1)
    return dict(best, cached=False, timings=entry["timings_ms_per_step"])
