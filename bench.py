#!/usr/bin/env python
"""Benchmark of the GB300-native Nyx PM step.

Headline workload (the plain GPU configuration): 256^3 dark-matter particles on
a 256^3 periodic grid, unit box, Einstein-de Sitter, seeded Zel'dovich ICs with
P(k) ~ k^-2 (rms displacement 0.2 cell at a = 0.02), FP64, a from 0.02 to 0.5 in
50 equal-delta-a steps.  A step is one full PM step of
Nyx::advance_particles_only (old-time deposit + solve, kick-drift, new-time
deposit + solve, kick) -- W warm-up steps then K timed steps of that schedule.

  python bench.py [--gpus N] [--steps K] [--warmup W] [--impl ours|reference]

One JSON line on rank 0.  N > 1 runs N independent replicas (one box per GPU,
no collective on the data path): weak scaling.
"""
from __future__ import annotations

import argparse
import json
import math
import os
import statistics
import subprocess
import sys
import threading
import time

REPO = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, REPO)

METRIC = "particle-steps/s per PM step"
UNIT = "particle-steps/s"
A_START, A_END, NSTEPS_CFG = 0.02, 0.5, 50


def parse():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=47)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", choices=["ours", "reference"], default="ours")
    ap.add_argument("--n", type=int, default=256)
    ap.add_argument("--no-cpu-baseline", action="store_true")
    ap.add_argument("--no-e2e", action="store_true")
    ap.add_argument("--no-ensemble", action="store_true")
    ap.add_argument("--no-serving", action="store_true")
    ap.add_argument("--no-c3", action="store_true",
                    help="skip the 512^3 mixed-precision object (c3)")
    ap.add_argument("--serving-requests", type=int, default=0,
                    help="requests in the serving stream (0: as many as ~60 s at 80%% load, "
                         "at most the configuration's 2000)")
    ap.add_argument("--ensemble-boxes", type=int, default=256)
    ap.add_argument("--ensemble-only", action="store_true",
                    help="run the batched-ensemble form alone and print its object (the command "
                         "the ensemble's ncu captures run)")
    ap.add_argument("--ensemble-steps", type=int, default=20)
    ap.add_argument("--tuning", type=str, default="",
                    help="deposit_tile,smooth_rows,inner_vcycles,sort_bucket[,prolong_quad] for the ensemble "
                         "instead of the autotuner's choice")
    ap.add_argument("--fused-edge", type=int, default=None,
                    help="nyxpm_params.mg_fused_edge: FP32 V-cycle levels of at most this many "
                         "(FP64: half as many) "
                         "cells per edge run as one CTA per box (default: the library's)")
    ap.add_argument("--quick", action="store_true",
                    help="headline timing only (no reuse-field pass, e2e or CPU baseline); "
                         "the command the ncu captures run")
    ap.add_argument("--accuracy", action="store_true",
                    help="mixed-precision accuracy report instead of the timing line: 512^3 "
                         "particles, P(k)~k^-2.5, 50 steps; relative L2 of rho, phi, g, x, v "
                         "of the mixed form against the FP64 form at steps 1, 10 and 50")
    ap.add_argument("--precision", choices=["fp64", "mixed"], default="fp64",
                    help="with --quick: the form the headline box uses (profiling the mixed "
                         "kernels); the default run always times FP64 first")
    ap.add_argument("--fraction", type=float, default=1.0,
                    help="with --quick: particles per cell (profiling the grid kernels of a "
                         "larger grid within a few GB)")
    ap.add_argument("--no-amr", action="store_true",
                    help="skip the multilevel (AMR) step object")
    ap.add_argument("--amr-only", action="store_true",
                    help="only the multilevel (AMR) step object, as its own JSON line")
    ap.add_argument("--amr-n0", type=int, default=128,
                    help="base grid of the multilevel workload (each level holds n0^3 cells)")
    ap.add_argument("--accuracy-n", type=int, default=512)
    ap.add_argument("--accuracy-steps", type=str, default="1,10,50")
    a = ap.parse_args()
    if a.quick:
        a.no_cpu_baseline = a.no_e2e = a.no_reuse = a.no_ensemble = a.no_serving = a.no_c3 = True
        a.no_amr = True
    else:
        a.no_reuse = False
        if a.precision != "fp64" or a.fraction != 1.0:
            ap.error("--precision and --fraction apply to --quick runs only")
    return a


def workload_config(n, W, K):
    return {
        "workload": f"plain PM FP64 drop-in: {n}^3 particles on a {n}^3 periodic grid, unit box, "
                    f"EdS h=0.675, Zel'dovich ICs P(k)~k^-2 seed 2, a {A_START}->{A_END} in "
                    f"{NSTEPS_CFG} equal-da steps; reference schedule (old- and new-time deposit "
                    f"+ solve per step), MG rel tol 1e-10",
        "n_grid": n,
        "n_particles": n ** 3,
        "steps_timed": f"schedule steps {W + 1}..{W + K}",
        "l2": "inputs larger than L2 (particle state 48 B x 16.7M = 805 MB, fields 128 MB each)",
        "parallelism": "replicas (one independent box per GPU)",
    }


def schedule(ctx_or_none, n_total):
    """Equal-da schedule of the workload; extends past a=0.5 with the same da if
    more steps are requested."""
    da = (A_END - A_START) / NSTEPS_CFG
    a_end = A_START + da * max(n_total, 1)
    if ctx_or_none is not None:
        return ctx_or_none.step_schedule(A_START, a_end, max(n_total, 1))
    from tests.pm_cases import equal_da_schedule
    return equal_da_schedule(A_START, a_end, max(n_total, 1))


# ---------------------------------------------------------------------------
# distributed plumbing (replicas: barrier + max-time reduction only)
# ---------------------------------------------------------------------------
def dist_env():
    ws = int(os.environ.get("WORLD_SIZE", "1"))
    rank = int(os.environ.get("RANK", "0"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    return ws, rank, local


def dist_init(backend):
    ws, rank, local = dist_env()
    if ws > 1:
        import torch.distributed as dist
        os.environ.setdefault("MASTER_ADDR", "127.0.0.1")
        dist.init_process_group(backend=backend)
    return ws, rank, local


def barrier(ws):
    if ws > 1:
        import torch.distributed as dist
        dist.barrier()


def allreduce_max(ws, v, device=None):
    if ws <= 1:
        return v
    import torch
    import torch.distributed as dist
    t = torch.tensor([v], dtype=torch.float64, device=device)
    dist.all_reduce(t, op=dist.ReduceOp.MAX)
    return float(t.item())


def allreduce_sum(ws, v, device=None):
    if ws <= 1:
        return v
    import torch
    import torch.distributed as dist
    t = torch.tensor([v], dtype=torch.float64, device=device)
    dist.all_reduce(t, op=dist.ReduceOp.SUM)
    return float(t.item())


def whole_job_rate(ws, units, ms, device=None):
    """Replicas: every rank timed its own units over the same barrier-bracketed
    region; the job rate is all ranks' units over the slowest rank's time.
    Returns (units per second, max ms)."""
    ms_max = allreduce_max(ws, ms, device)
    total = allreduce_sum(ws, float(units), device)
    return total / (ms_max / 1e3), ms_max


def replica_seed(rank):
    """Each replica advances its own box: the workload's seed 2, shifted by rank."""
    return 2 + rank


# ---------------------------------------------------------------------------
# clocks during the timed region
# ---------------------------------------------------------------------------
class ClockSampler:
    FIELDS = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
              "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
              "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self, device_index):
        self.lines = []
        self.proc = None
        cmd = ["nvidia-smi", f"--query-gpu={self.FIELDS}", "--format=csv,noheader,nounits", "-lms", "200"]
        sel = self._selector(device_index)
        if sel:
            cmd += ["-i", sel]
        try:
            self.proc = subprocess.Popen(cmd, stdout=subprocess.PIPE, stderr=subprocess.DEVNULL, text=True)
            self.thread = threading.Thread(target=self._read, daemon=True)
            self.thread.start()
        except Exception:
            self.proc = None

    @staticmethod
    def _selector(device_index):
        try:
            import torch
            u = str(torch.cuda.get_device_properties(device_index).uuid)
            return u if u.startswith("GPU-") else "GPU-" + u
        except Exception:
            return None

    def _read(self):
        for line in self.proc.stdout:
            self.lines.append(line.strip())

    def stop(self):
        if self.proc is None:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["nvidia-smi unavailable"]}
        time.sleep(0.25)
        self.proc.terminate()
        try:
            self.proc.wait(timeout=5)
        except Exception:
            self.proc.kill()
        sm, smax, power, reasons = [], [], [], set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        for ln in self.lines:
            parts = [p.strip() for p in ln.split(",")]
            if len(parts) < 9:
                continue
            try:
                sm.append(float(parts[1]))
                smax.append(float(parts[2]))
                power.append(float(parts[3]))
            except ValueError:
                continue
            for nm, v in zip(names, parts[5:9]):
                if v.lower() == "active":
                    reasons.add(nm)
        return {"sm_mhz": statistics.median(sm) if sm else None,
                "sm_max_mhz": max(smax) if smax else None,
                "power_w_max": max(power) if power else None,
                "samples": len(sm), "reasons": sorted(reasons)}


def measured_peaks():
    p = os.path.join(REPO, "MEASURED_PEAKS.json")
    if os.path.exists(p):
        with open(p) as f:
            d = json.load(f)
        return float(d["hbm_gbs"]), "measured"
    return 6800.0, "fallback"


def ncu_traffic():
    """Per-launch DRAM bytes of the dominant kernels from the committed ncu summary."""
    p = os.path.join(REPO, "profiles", "ncu_traffic.json")
    if os.path.exists(p):
        with open(p) as f:
            return json.load(f)
    return {}


# ---------------------------------------------------------------------------
# the CPU oracle (baseline arm)
# ---------------------------------------------------------------------------
def oracle_steps(ic, sched, n, max_seconds, pm=None):
    """Run oracle PM steps (from the ICs, or continuing pm) until the schedule or
    the time budget is exhausted; returns (steps_done, seconds, threads, pm)."""
    from oracle import oracle as O
    if pm is None:
        p = O.Particles(ic.pos, ic.vel, ic.mass)
        pm = O.PMOracle(n, ic.L, p)
    done, secs = 0, 0.0
    for a0, a1, dt in sched:
        t0 = time.perf_counter()
        pm.step(a0, a1, dt)
        secs += time.perf_counter() - t0
        done += 1
        if secs >= max_seconds:
            break
    return done, secs, O.num_threads(), pm


# ---------------------------------------------------------------------------
# ensemble and serving forms
# ---------------------------------------------------------------------------
def _ic_worker(args):
    from nyx_gb300.ics import zeldovich_ics
    n, L, slope, seed, a, frac = args
    ic = zeldovich_ics(n, L, slope, seed, a, rms_disp_cells=0.2, fraction=frac)
    return ic.pos, ic.vel, ic.mass


def make_ics(jobs):
    """Seeded ICs for many boxes, generated by a spawn process pool (host FFTs)."""
    import multiprocessing as mp
    procs = max(1, min(len(jobs), (os.cpu_count() or 2) - 2))
    with mp.get_context("spawn").Pool(procs) as pool:
        return pool.map(_ic_worker, jobs, chunksize=1)


def rel_l2(a, b):
    import numpy as np
    a = np.asarray(a, dtype=np.float64).ravel()
    b = np.asarray(b, dtype=np.float64).ravel()
    return float(np.linalg.norm(a - b) / np.linalg.norm(b))


def plain_fp64_run(ctx, n, L, pos, vel, mass, sched, stream):
    """The plain FP64 drop-in on one box, on the ensemble's schedule (the post_init
    solve at the first a, then one deposit + solve per step, the old-time field
    reused): device ms by CUDA events on the library stream, and the box (open)."""
    import torch
    from nyx_gb300.pm import Box
    box = Box(ctx, n, L, len(pos))
    box.upload(pos, vel, mass)
    e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    e0.record(stream)
    box.init_field(sched[0][0])
    for a0, a1, dt in sched:
        box.step(a0, a1, dt, reuse_field=True)
    e1.record(stream)
    e1.synchronize()
    return e0.elapsed_time(e1), box


def run_ensemble_form(ctx, nboxes, steps=20, fixed_tuning=None, stream=None):
    """Batched ensemble: 256 boxes of {32..128}^3, particles = cells x {0.5, 1},
    slopes in [-2.5, -1.5], a 0.02 -> 0.2 in 20 steps, mixed precision, one
    persistent launch per stage, captured step graphs, autotuned shapes.  The
    comparison is the plain FP64 drop-in on the same boxes, ICs and schedule, one
    box at a time, measured; the force error of each box is its gravity vector
    after the 20 steps against the FP64 box's (both free running from the same
    ICs)."""
    import numpy as np
    from nyx_gb300 import autotune
    from nyx_gb300.ensemble import Ensemble, ensemble_workload
    specs = ensemble_workload(nboxes, seed=4)
    t0 = time.perf_counter()
    ics = make_ics([(s.n, s.L, s.slope, s.seed, A_START, s.fraction) for s in specs])
    t_ic = time.perf_counter() - t0
    by_id = {id(s): ic for s, ic in zip(specs, ics)}
    if fixed_tuning:
        tune = dict(dict(zip(("deposit_tile", "smooth_rows", "inner_vcycles", "sort_bucket", "prolong_quad"),
                             fixed_tuning)),
                    cached=True)
    else:
        tune = autotune.tune(ctx, specs,
                             cache_path=os.path.join(REPO, "nyx_gb300", "_tuning_cache.json"),
                             ic_provider=lambda s: by_id[id(s)])
    arena = int(sum(Ensemble.box_bytes(s.n, s.np) for s in specs) * 1.05) + (256 << 20)
    ens = Ensemble(ctx, arena)
    tune.setdefault("sort_bucket", 256)
    tune.setdefault("prolong_quad", 1)
    knobs = ("deposit_tile", "smooth_rows", "inner_vcycles", "sort_bucket", "prolong_quad")
    ens.set_tuning(**{k: tune[k] for k in knobs})
    slots = []
    for s, (pos, vel, mass) in zip(specs, ics):
        slot = ens.add(s.n, s.L, s.np)
        ens.upload(slot, pos, vel, mass)
        slots.append(slot)
    sched = ctx.step_schedule(A_START, 0.2, steps)
    total_ms, infos = 0.0, []
    launches0 = ctx.launch_count()
    for a0, a1, dt in sched:
        info = ens.step({q: a0 for q in slots}, {q: a1 for q in slots}, {q: dt for q in slots})
        total_ms += info["ms"]
        infos.append(info)
    launches = ctx.launch_count() - launches0
    # the plain FP64 drop-in on the same boxes and schedule, one box at a time
    # (CUDA events around each box's run), and each box's force error
    plain_ms, ferr = 0.0, []
    for s, slot, (pos, vel, mass) in zip(specs, slots, ics):
        ms_b, box = plain_fp64_run(ctx, s.n, s.L, pos, vel, mass, sched, stream)
        plain_ms += ms_b
        ferr.append(rel_l2(ens.grav_vector(slot), box.grav_vector()))
        box.close()
    ferr = np.asarray(ferr)
    # per-stage CUDA-event times of two more steps run eagerly (outside the timed region)
    a_last = sched[-1][1]
    ctx.set_profiling(True)
    ctx.profile(reset=True)
    for a0, a1, dt in ctx.step_schedule(a_last, a_last + 0.018, 2):
        ens.step({q: a0 for q in slots}, {q: a1 for q in slots}, {q: dt for q in slots})
    eprof = ctx.profile(reset=True)
    ctx.set_profiling(False)
    etot = sum(v["ms"] for v in eprof["stages"].values()) or 1.0
    estages = {k: {"launches": v["launches"], "ms": round(v["ms"], 3),
                   "share": round(v["ms"] / etot, 3)}
               for k, v in eprof["stages"].items() if v["launches"]}
    ens.close()
    psteps = sum(s.np for s in specs) * steps
    steady = [i["ms"] for i in infos[1:]]
    return {
        "boxes": nboxes, "steps": steps, "particles": int(sum(s.np for s in specs)),
        "cells": int(sum(s.n ** 3 for s in specs)),
        "size_mix": autotune.signature(specs),
        "value": psteps / (total_ms / 1e3), "unit": UNIT,
        "runs_per_s": nboxes / (total_ms / 1e3), "total_s": total_ms / 1e3,
        "steady_ms_per_step": float(np.mean(steady)) if steady else None,
        "first_step_ms_incl_initial_solve_and_capture": infos[0]["ms"],
        "max_outer_iters": max(i["max_outer_used"] for i in infos),
        "fallback_iters": sum(i["fallback_iters"] for i in infos),
        "launches_per_step": launches / steps,
        "tuning": {k: tune[k] for k in knobs},
        "tuning_cached": tune.get("cached", False),
        "plain_fp64_same_schedule": {
            "value": psteps / (plain_ms / 1e3), "unit": UNIT, "total_s": plain_ms / 1e3,
            "runs_per_s": nboxes / (plain_ms / 1e3),
            "note": "the FP64 drop-in on the same 256 boxes, ICs and schedule (post_init solve, "
                    "then one deposit + solve per step), one box at a time; CUDA events "
                    "around each box's run, summed: measured, not extrapolated"},
        "speedup_vs_plain_fp64_same_schedule": plain_ms / total_ms,
        "force_rel_l2_vs_fp64": {"worst_box": float(ferr.max()), "median_box": float(np.median(ferr)),
                                 "boxes": int(len(ferr)),
                                 "measure": "relative L2 of the gravity vector after the 20 steps, "
                                            "mixed ensemble box against the FP64 box run from the "
                                            "same ICs on the same schedule (free running)"},
        "ic_generation_s": t_ic,
        "stages_eager_2_steps": estages,
    }


def run_serving_form(ctx, nreq_arg, tuning=None, budget_gb=150.0):
    """Serving: Poisson arrivals at ~80% of measured capacity, n in {32..192}^3
    (weights 30/25/20/12/8/5 %), 10-40 steps, 150 GB HBM budget, continuous
    batching.  The comparison is the plain FP64 drop-in serving one run at a time on
    the same step schedule:
      * capacity against capacity: both servers with every request available at once;
      * latency at one offered load both can carry: a stream at 80 % of the FP64
        server's capacity served by each, p50/p99 of both;
      * accuracy: on a sample of that stream's runs, the relative L2 of the final
        gravity vector of the mixed server's run against the FP64 server's run of
        the same request (both free running from the same ICs)."""
    import numpy as np
    from nyx_gb300.serving import ContinuousBatchingServer, request_stream, serve_sequential, SIZES
    # IC pool: 6 seeded ICs per size (distinct seeds and slopes); request r uses entry r mod 6
    rng = np.random.default_rng(55)
    jobs, keys = [], []
    for n in SIZES:
        for j in range(6):
            jobs.append((n, 1.0, float(rng.uniform(-2.5, -1.5)), int(rng.integers(1, 2 ** 31 - 1)),
                         0.02, 1.0))
            keys.append((n, j))
    pool = dict(zip(keys, make_ics(jobs)))

    class IC:
        def __init__(self, t):
            self.pos, self.vel, self.mass = t

    def provider(r):
        return IC(pool[(r.n, r.rid % 6)])

    budget = int(budget_gb * 1e9)
    # capacity: a burst of requests all available at t = 0
    burst = request_stream(200, 0.0, seed=6)
    srv = ContinuousBatchingServer(ctx, budget, provider, tuning=tuning)
    capacity = srv.serve(burst, realtime=False).summary()["runs_per_s"]
    rate = 0.8 * capacity
    nreq = nreq_arg or int(min(2000, max(100, 60.0 * rate)))
    reqs = request_stream(nreq, rate, seed=5)
    s_sum = srv.serve(reqs, realtime=True).summary()
    # the FP64 server's capacity on the same burst's first 60 requests (same schedule)
    seq_cap = serve_sequential(ctx, burst[:60], provider, realtime=False).summary()["runs_per_s"]
    # both servers at one offered load below both capacities: 80 % of the FP64 server's
    rate_same = 0.8 * seq_cap
    same = request_stream(int(max(40, min(100, 20.0 * rate_same))), rate_same, seed=7)
    sample = {r.rid for r in same[::4]}
    srv.keep = sample
    m_same = srv.serve(same, realtime=True)
    srv.close()
    q_same = serve_sequential(ctx, same, provider, realtime=True, keep_results=sample)
    gm = {r.rid: r.g for r in m_same.results if r.g is not None}
    errs = np.asarray([rel_l2(gm[r.rid], r.g) for r in q_same.results if r.g is not None and r.rid in gm])
    ms_, qs_ = m_same.summary(), q_same.summary()
    return {
        "requests": nreq, "requests_in_config": 2000, "arrival_rate_per_s": rate,
        "measured_capacity_runs_per_s": capacity, "budget_GB": budget_gb,
        "runs_per_s": s_sum["runs_per_s"], "p50_latency_s": s_sum["p50_latency_s"],
        "p99_latency_s": s_sum["p99_latency_s"], "max_concurrent_runs": s_sum["max_concurrent_runs"],
        "peak_arena_GB": s_sum["peak_arena_GB"], "particle_steps_per_s": s_sum["particle_steps_per_s"],
        "capacity_vs_plain_fp64": {
            "mixed_server_runs_per_s": capacity, "plain_fp64_runs_per_s": seq_cap,
            "ratio": capacity / seq_cap if seq_cap else None,
            "note": "every request available at once (200-request burst; the FP64 server its "
                    "first 60), both on the same schedule (post_init solve, then one deposit + "
                    "solve per step)"},
        "same_offered_load": {
            "arrival_rate_per_s": rate_same, "requests": len(same),
            "mixed_server": {"runs_per_s": ms_["runs_per_s"], "p50_latency_s": ms_["p50_latency_s"],
                             "p99_latency_s": ms_["p99_latency_s"]},
            "plain_fp64_one_at_a_time": {"runs_per_s": qs_["runs_per_s"],
                                         "p50_latency_s": qs_["p50_latency_s"],
                                         "p99_latency_s": qs_["p99_latency_s"]},
            "p50_latency_ratio": (qs_["p50_latency_s"] / ms_["p50_latency_s"]
                                  if ms_["p50_latency_s"] else None),
            "note": "one Poisson stream at 80 % of the FP64 server's capacity, so neither "
                    "queue grows without bound; latency = completion - arrival"},
        "force_rel_l2_vs_fp64": {"worst_run": float(errs.max()) if errs.size else None,
                                 "median_run": float(np.median(errs)) if errs.size else None,
                                 "runs": int(errs.size),
                                 "measure": "final gravity vector of a run served in the mix against "
                                            "the FP64 server's run of the same request (every 4th "
                                            "request of the same-load stream)"},
        "note": "ICs from a pool of 6 seeded ICs per size",
    }


def run_c3_form(ctx, stream, n=512, steps=NSTEPS_CFG):
    """The mixed-precision configuration at full size: 512^3 particles on a 512^3 grid,
    P(k) ~ k^-2.5, seed 3, a 0.02 -> 0.5 in 50 equal-da steps on Nyx's two-solve
    schedule.  The FP64 drop-in runs the same ICs and schedule in lockstep on a box
    of its own; each step of each form is timed by its own CUDA event pair, and at
    steps 1, 10 and 50 the relative L2 of the mixed form's rho, phi, g, x and v
    against the FP64 form's is taken (free running from the same ICs; at step 1
    that is one mixed step from the FP64 state)."""
    import numpy as np
    import torch
    from nyx_gb300.ics import zeldovich_ics
    from nyx_gb300.pm import Box
    t0 = time.perf_counter()
    ic = zeldovich_ics(n, 1.0, -2.5, 3, A_START, rms_disp_cells=0.2,
                       device=f"cuda:{torch.cuda.current_device()}")
    t_ic = time.perf_counter() - t0
    npart = len(ic.pos)
    sched = ctx.step_schedule(A_START, A_END, steps)
    bm = Box(ctx, n, 1.0, npart, precision="mixed")
    bf = Box(ctx, n, 1.0, npart)
    bm.upload(ic.pos, ic.vel, ic.mass)
    bf.upload(ic.pos, ic.vel, ic.mass)
    e = [torch.cuda.Event(enable_timing=True) for _ in range(4)]
    ms_m = ms_f = 0.0
    rows, outer = [], []

    def mr(f):
        return f - f.mean()

    def minimg(d):
        return (d + 0.5) % 1.0 - 0.5

    for k, (a0, a1, dt) in enumerate(sched, start=1):
        e[0].record(stream)
        info = bm.step(a0, a1, dt)
        e[1].record(stream)
        bf.step(a0, a1, dt)
        e[2].record(stream)
        e[2].synchronize()
        ms_m += e[0].elapsed_time(e[1])
        ms_f += e[1].elapsed_time(e[2])
        outer.append(info["new_solve"]["vcycles"])
        if k in (1, 10, steps):
            row = {"step": k, "a": a1, "rho": rel_l2(bm.deposit(), bf.deposit()),
                   "phi": rel_l2(mr(bm.get_phi()), mr(bf.get_phi())),
                   "g": rel_l2(bm.grav_vector(), bf.grav_vector())}
            pm_, vm_ = bm.download()
            pf_, vf_ = bf.download()
            row["x"] = float(np.linalg.norm(minimg(pm_ - pf_)) / np.linalg.norm(minimg(pf_ - ic.lattice)))
            row["v"] = rel_l2(vm_, vf_)
            rows.append(row)
    bm.close()
    bf.close()
    del ic
    psteps = float(npart) * steps
    return {
        "workload": f"{n}^3 particles on a {n}^3 periodic grid, unit box, Zel'dovich ICs P(k)~k^-2.5 "
                    f"seed 3, a {A_START}->{A_END} in {steps} equal-da steps, reference schedule "
                    f"(two deposits + solves per step), MG rel tol 1e-10",
        "n_grid": n, "n_particles": npart, "steps": steps,
        "value": psteps / (ms_m / 1e3), "unit": UNIT, "ms_per_step": ms_m / steps,
        "plain_fp64_same_schedule": {"value": psteps / (ms_f / 1e3), "unit": UNIT,
                                     "ms_per_step": ms_f / steps},
        "speedup_vs_plain_fp64_same_schedule": ms_f / ms_m,
        "outer_iters_new_solve_mean": float(np.mean(outer)),
        "force_rel_l2_vs_fp64": max(r["g"] for r in rows),
        "errors_vs_fp64": rows,
        "ic_generation_s": t_ic,
        "note": "both forms step the same ICs on the same schedule in lockstep, each step timed "
                "by its own CUDA event pair on the library stream; errors: relative L2 of the "
                "mixed form against the FP64 form (which equals the FP64 oracle bit for bit in the "
                "parity tests), free running; x as displacement from the lattice, minimum image",
    }


def amr_workload(n0, seed=7):
    """A zoom-shaped multilevel workload: n0^3 Zel'dovich particles (P(k)~k^-2,
    rms displacement 0.2 cell at a = 0.02) plus n0^3/8 particles in a Gaussian
    cluster (sigma 0.1, central overdensity about 8) at the centre with
    velocities of the same spread (clipped at 2.5 sigma), equal masses; level 1
    refines [0.25, 0.75)^3 and level 2 [0.375, 0.625)^3 (one box each, n0^3
    cells each)."""
    import numpy as np
    from nyx_gb300.ics import zeldovich_ics
    ic = zeldovich_ics(n0, 1.0, -2.0, seed, A_START, rms_disp_cells=0.2)
    rng = np.random.default_rng(seed)
    nc = n0 ** 3 // 8
    sig = float(np.std(ic.vel))
    pos = np.concatenate([ic.pos, (0.5 + rng.normal(0, 0.1, (nc, 3))) % 1.0])
    vel = np.concatenate([ic.vel, np.clip(rng.normal(0, sig, (nc, 3)), -2.5 * sig, 2.5 * sig)])
    boxes = [[((n0 // 2,) * 3, (3 * n0 // 2 - 1,) * 3)], [((3 * n0 // 2,) * 3, (5 * n0 // 2 - 1,) * 3)]]
    return pos, vel, float(ic.mass), boxes


AMR_A_END, AMR_STEPS = 0.04, 40


def run_amr_form(ctx, stream, n0=128, warmup=2, timed=10, cpu_n0=64, cpu_seconds=20.0):
    """The multilevel step without subcycling (nyxpm_amr_step) on amr_workload(n0):
    warmup + timed steps of a 0.02 -> 0.04 in 40 equal-da steps, each timed by a
    CUDA event pair on the library stream, then one profiled step for the
    smoothers' FP64 roofline; the CPU oracle of the same step on the
    same-shaped workload at n0 = cpu_n0 as a bounded sample."""
    import numpy as np
    import torch
    from nyx_gb300.amr import AmrHierarchy
    from oracle import oracle as O
    pos, vel, mass, boxes = amr_workload(n0)
    npart = len(pos)
    H = AmrHierarchy(ctx, n0, 1.0, boxes, npart)
    H.upload(pos, vel, mass)
    lev, _ = H.assign()
    per_level = np.bincount(lev, minlength=3).tolist()
    sched = ctx.step_schedule(A_START, AMR_A_END, AMR_STEPS)
    e = [torch.cuda.Event(enable_timing=True) for _ in range(2)]
    ms, vc, launches = [], [], 0
    for k, (a0, a1, dt) in enumerate(sched[:warmup + timed]):
        l0 = ctx.launch_count()
        e[0].record(stream)
        info = H.step(a0, a1, dt)
        e[1].record(stream)
        e[1].synchronize()
        if k >= warmup:
            ms.append(e[0].elapsed_time(e[1]))
            vc.append((info["old_solve"]["vcycles"], info["new_solve"]["vcycles"]))
            launches += ctx.launch_count() - l0
    # one more step with per-launch events: the red-black half sweeps of every
    # level (k_amr_gsrbf on the fine levels, k_gsrb on level 0's hierarchy) against
    # the FP64 rates of this GPU, as the headline's roofline does
    ctx.set_profiling(True)
    ctx.profile(reset=True)
    H.step(*sched[warmup + timed])
    prof = ctx.profile(reset=True)
    ctx.set_profiling(False)
    fs = prof["fine_smooth"]
    stage_ms = sum(v["ms"] for v in prof["stages"].values())
    fp64_peak, fp64_add = ctx.measure_fp64_peak()
    updates = fs["bytes"] / 24.0
    ops = 6.0 * updates / (fs["ms"] * 1e-3) / 1e12
    peak_ops = 6.0 / (5.0 / fp64_add + 1.0 / (fp64_peak / 2.0))
    roofline = {"bound": "fp64", "kernel": "red-black half sweeps of every level (k_amr_gsrbf, level 0's k_gsrb)",
                "achieved": round(ops, 4), "peak": round(peak_ops, 4), "frac": round(ops / peak_ops, 4),
                "unit": "T FP64 op/s (an add or an FMA is one op; 6 per updated cell)",
                "peak_source": "measured: nyxpm_measure_fp64_peak on this GPU, weighted 5 adds : 1 FMA",
                "launches": fs["launches"], "ms": round(fs["ms"], 3),
                "share_of_step": round(fs["ms"] / stage_ms, 3) if stage_ms > 0 else None}
    H.close()
    # the oracle (all host threads) on the same-shaped workload at cpu_n0
    cpos, cvel, cmass, cboxes = amr_workload(cpu_n0)
    p = O.Particles(cpos, cvel, cmass)
    A = O.AmrOracle(cpu_n0, 1.0, cboxes, p)
    done, secs = 0, 0.0
    for a0, a1, dt in sched:
        t0 = time.perf_counter()
        A.step(a0, a1, dt)
        secs += time.perf_counter() - t0
        done += 1
        if secs >= cpu_seconds:
            break
    tot = sum(ms)
    cells = [n0 ** 3, n0 ** 3, n0 ** 3]
    return {
        "workload": f"{n0}^3 Zel'dovich particles (P(k)~k^-2) + {n0 ** 3 // 8} in a central Gaussian "
                    f"cluster, base grid {n0}^3, level 1 [0.25,0.75)^3 and level 2 [0.375,0.625)^3 "
                    f"({n0}^3 cells each, ratio 2), a {A_START}->{AMR_A_END} in {AMR_STEPS} equal-da "
                    f"steps, no subcycling, two multilevel solves per step from phi = 0, rel tol 1e-10",
        "n_particles": npart, "particles_per_level": per_level, "cells_per_level": cells,
        "steps": timed, "warmup": warmup,
        "value": npart * timed / (tot / 1e3), "unit": UNIT, "ms_per_step": tot / timed,
        "vcycles_per_solve_mean": float(np.mean(vc)), "launches_per_step": launches / timed,
        "dtype": "f64", "roofline": roofline,
        "cpu_baseline": {"value": len(cpos) * done / secs, "unit": UNIT, "cores": O.num_threads(),
                         "kind": "port", "seconds": secs,
                         "sample": f"{done} steps of the same-shaped workload at base grid {cpu_n0}^3 "
                                   f"({len(cpos)} particles), the multilevel C++/OpenMP oracle on "
                                   f"{O.num_threads()} host threads"},
        "note": "each step timed by its own CUDA event pair on the library stream; the solves read "
                "their residual norm on the host after every composite V-cycle",
    }


def run_amr_only(args):
    import torch
    from nyx_gb300 import _lib
    _lib.load()
    from nyx_gb300.pm import Context
    ctx = Context(device=0)
    stream = torch.cuda.ExternalStream(ctx.stream, device=torch.device("cuda", 0))
    out = run_amr_form(ctx, stream, n0=args.amr_n0)
    ctx.close()
    print(json.dumps({"amr": out}), flush=True)
    return 0


def run_reference(args):
    ws, rank, _ = dist_init("gloo")
    if rank != 0:
        return 0
    from nyx_gb300.ics import zeldovich_ics
    from oracle import oracle as O
    O.build()
    n = args.n
    ic = zeldovich_ics(n, 1.0, -2.0, 2, A_START, rms_disp_cells=0.2)
    sched = schedule(None, args.warmup + args.steps)
    # warm-up: one step (bounded), then timed steps within a ~150 s budget
    w = min(args.warmup, 1)
    pm = None
    if w:
        _, _, _, pm = oracle_steps(ic, sched[:1], n, 1e9)
    done, secs, threads, _ = oracle_steps(ic, sched[w:w + args.steps], n, 150.0, pm)
    value = n ** 3 * done / secs
    sample = (f"{done} of the {args.steps} timed steps (steps {w + 1}..{w + done} of the schedule), "
              f"each a full FP64 PM step of the {n}^3 workload, C++/OpenMP oracle")
    line = {
        "impl": "reference", "metric": METRIC, "value": value, "unit": UNIT, "n_gpus": args.gpus,
        "steps": args.steps, "warmup": args.warmup, "ms_per_step": 1e3 * secs / done,
        "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f64",
        "data": "synthetic", "config": workload_config(n, args.warmup, args.steps),
        "cpu_baseline": {"value": value, "unit": UNIT, "cores": threads, "kind": "port",
                         "sample": sample},
        "e2e": {"value": value, "unit": UNIT, "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0},
        "note": "Nyx's own CPU PM step needs AMReX (absent from the reference tree); the arm times "
                "the FP64 C++/OpenMP restatement of it on all host cores",
    }
    print(json.dumps(line), flush=True)
    return 0


# ---------------------------------------------------------------------------
# our arm
# ---------------------------------------------------------------------------
def run_ours(args):
    import numpy as np
    import torch
    ws, rank, local = dist_init("nccl")
    torch.cuda.set_device(local)
    from nyx_gb300 import _lib
    _lib.load()
    from nyx_gb300.ics import zeldovich_ics
    from nyx_gb300.pm import Box, Context

    n = args.n
    W, K = args.warmup, args.steps
    ic = zeldovich_ics(n, 1.0, -2.0, replica_seed(rank), A_START, rms_disp_cells=0.2,
                       fraction=args.fraction)
    npart = len(ic.pos)
    ctx = Context(device=local, mg_fused_edge=args.fused_edge)
    stream = torch.cuda.ExternalStream(ctx.stream, device=torch.device("cuda", local))
    sched = schedule(ctx, W + K)
    box = Box(ctx, n, 1.0, npart, precision=args.precision)
    box.upload(ic.pos, ic.vel, ic.mass)

    # ---- the FP64 issue rate of this GPU (outside the timed region): the
    #      denominator of the FP64 form's roofline ----
    fp64_peak, fp64_add = ctx.measure_fp64_peak() if args.precision == "fp64" else (None, None)

    # ---- device-resident run: warm-up, then K timed steps (solver iterations
    #      replayed from the box's CUDA graphs) ----
    for a0, a1, dt in sched[:W]:
        box.step(a0, a1, dt)
    vcycles = []
    launches0 = ctx.launch_count()
    clocks = ClockSampler(local)
    barrier(ws)
    torch.cuda.synchronize()
    e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    e0.record(stream)
    for a0, a1, dt in sched[W:W + K]:
        info = box.step(a0, a1, dt)
        vcycles.append((info["old_solve"]["vcycles"], info["new_solve"]["vcycles"]))
    e1.record(stream)
    torch.cuda.synchronize()
    barrier(ws)
    clk = clocks.stop()
    launches = ctx.launch_count() - launches0
    ms = e0.elapsed_time(e1)
    value, ms_max = whole_job_rate(ws, float(npart) * K, ms, torch.device("cuda", local))

    # ---- the same W + K steps again from the same ICs, the K steps with a CUDA
    #      event pair around every launch (eager launches): the stage split and
    #      the dominant kernel's launch durations ----
    box.upload(ic.pos, ic.vel, ic.mass)
    for a0, a1, dt in sched[:W]:
        box.step(a0, a1, dt)
    ctx.set_profiling(True)
    ctx.profile(reset=True)
    torch.cuda.synchronize()
    e0.record(stream)
    for a0, a1, dt in sched[W:W + K]:
        box.step(a0, a1, dt)
    e1.record(stream)
    torch.cuda.synchronize()
    ms_profiled = e0.elapsed_time(e1)
    prof = ctx.profile(reset=True)
    ctx.set_profiling(False)

    # ---- roofline of the dominant kernel ----
    stages = prof["stages"]
    stage_rows = {k: {"launches": v["launches"], "ms": round(v["ms"], 3),
                      "GB/s": round(v["bytes"] / (v["ms"] * 1e6), 1) if v["ms"] > 0 else None}
                  for k, v in stages.items() if v["launches"]}
    dom = max(stages, key=lambda k: stages[k]["ms"])
    peak, peak_kind = measured_peaks()
    traffic = ncu_traffic()
    if dom == "smooth" and prof["fine_smooth"]["launches"]:
        fs = prof["fine_smooth"]
        per_launch = fs["bytes"] / fs["launches"]
        avg_ms = fs["ms"] / fs["launches"]
        kname = ("k_gsrb (finest-level FP64 red-black half sweep)" if args.precision == "fp64" else
                 "k_gsrb_f4 (finest-level FP32 red-black half sweep)")
        tr = traffic.get("k_gsrb_fine") if args.precision == "fp64" else None
    else:
        st = stages[dom]
        per_launch = st["bytes"] / max(st["launches"], 1)
        avg_ms = st["ms"] / max(st["launches"], 1)
        kname = dom
        tr = traffic.get(dom)
    achieved = per_launch / (avg_ms * 1e6)
    hbm = {"achieved": round(achieved, 1), "peak": peak, "peak_source": peak_kind, "unit": "GB/s",
           "frac": round(achieved / peak, 4)}
    share = round(stages[dom]["ms"] / sum(v["ms"] for v in stages.values()), 3)
    traffic_launch = tr * (n / traffic.get("n", n)) ** 3 if tr else None
    if args.precision == "fp64" and dom == "smooth" and prof["fine_smooth"]["launches"]:
        # the finest FP64 half sweep updates n^3/2 cells with 6 FP64 operations each
        # (5 additions of the neighbour sum and one fused multiply-add), 24 algorithmic
        # bytes per cell.  The bound is the time the FP64 pipe needs for that mix at the
        # rates measured on this GPU: 5 / add rate + 1 / FMA rate per cell, i.e. a peak
        # of 6 / (5 / R_add + 1 / R_fma) operations per second
        cells = per_launch / 24.0
        ops = 6.0 * cells / (avg_ms * 1e-3) / 1e12
        r_fma = fp64_peak / 2.0
        peak_ops = 6.0 / (5.0 / fp64_add + 1.0 / r_fma)
        roofline = {"bound": "fp64", "kernel": kname,
                    "achieved": round(ops, 4), "peak": round(peak_ops, 4),
                    "peak_source": "measured: nyxpm_measure_fp64_peak on this GPU (chains of FP64 "
                                   "additions and of FMAs, CUDA events), weighted 5 adds : 1 FMA",
                    "unit": "T FP64 op/s (an add or an FMA is one op)",
                    "frac": round(ops / peak_ops, 4), "traffic": traffic_launch,
                    "fp64_rates_measured": {"fma_T_per_s": round(r_fma, 4),
                                            "add_T_per_s": round(fp64_add, 4)},
                    "flops": {"achieved_TFLOPs": round(7.0 * cells / (avg_ms * 1e-3) / 1e12, 4),
                              "peak_TFLOPs": round(fp64_peak, 4),
                              "note": "FMA = 2 flops: 7 flops per updated cell; peak = FMA chains"},
                    "hbm": hbm,
                    "algorithmic_bytes_per_launch": per_launch, "avg_launch_ms": avg_ms,
                    "fp64_pipe_active_ncu": traffic.get("k_gsrb_fine_fp64_pipe_active"),
                    "dominant_stage_share": share}
    else:
        roofline = dict(hbm, bound="hbm", kernel=kname, traffic=traffic_launch,
                        algorithmic_bytes_per_launch=per_launch, avg_launch_ms=avg_ms,
                        dominant_stage_share=share)

    line = {
        "metric": METRIC, "value": value, "unit": UNIT, "n_gpus": ws, "steps": K, "warmup": W,
        "ms_per_step": ms_max / K, "higher_is_better": True, "scaling": "weak",
        "vs_baseline": None, "data": "synthetic",
        "dtype": "f64" if args.precision == "fp64" else "f32 (inside FP64 defect correction)",
        "config": workload_config(n, W, K),
        "roofline": roofline, "clocks": clk, "gpu_launches": int(launches),
        "stages": stage_rows,
        "profiled_replay_ms_per_step": ms_profiled / K,
        "profiling_note": ("stages and roofline: a second run of the same W + K steps from the "
                           "same ICs with a CUDA event pair around every launch, enqueued "
                           "eagerly; the timed run replays each solver iteration from a CUDA "
                           "graph"),
        "vcycles_per_step": {"old_mean": float(np.mean([v[0] for v in vcycles])),
                             "new_mean": float(np.mean([v[1] for v in vcycles]))},
    }

    if args.precision != "fp64" or args.fraction != 1.0:
        line["config"].update(precision=args.precision, fraction=args.fraction,
                              n_particles=npart, note="profiling run, not the headline workload")

    # ---- same workload with the old-time field reused (1 deposit + 1 solve per step) ----
    if not args.no_reuse:
        box.upload(ic.pos, ic.vel, ic.mass)
        box.init_field(A_START)
        for a0, a1, dt in sched[:W]:
            box.step(a0, a1, dt, reuse_field=True)
        torch.cuda.synchronize()
        e0.record(stream)
        for a0, a1, dt in sched[W:W + K]:
            box.step(a0, a1, dt, reuse_field=True)
        e1.record(stream)
        torch.cuda.synchronize()
        ms_r = allreduce_max(ws, e0.elapsed_time(e1), torch.device("cuda", local))
        line["reuse_field"] = {
            "value": allreduce_sum(ws, float(npart) * K, torch.device("cuda", local)) / (ms_r / 1e3),
            "ms_per_step": ms_r / K, "note": "old-time field taken from the previous new-time solve"}

    # ---- mixed precision (FP32 particles, FP32 deposit + V-cycles inside FP64 defect
    #      correction), old-time field reused: the optimised form of the same workload ----
    if not args.no_reuse:
        bm = Box(ctx, n, 1.0, npart, precision="mixed")
        bm.upload(ic.pos, ic.vel, ic.mass)
        bm.init_field(A_START)
        for a0, a1, dt in sched[:W]:
            bm.step(a0, a1, dt, reuse_field=True)
        torch.cuda.synchronize()
        minfo = []
        e0.record(stream)
        for a0, a1, dt in sched[W:W + K]:
            minfo.append(bm.step(a0, a1, dt, reuse_field=True)["new_solve"])
        e1.record(stream)
        torch.cuda.synchronize()
        ms_m = allreduce_max(ws, e0.elapsed_time(e1), torch.device("cuda", local))
        # per-stage CUDA-event times of three more steps (outside the timed region)
        a_last = sched[W + K - 1][1]
        da = (A_END - A_START) / NSTEPS_CFG
        ctx.set_profiling(True)
        ctx.profile(reset=True)
        for a0, a1, dt in ctx.step_schedule(a_last, a_last + 3 * da, 3):
            bm.step(a0, a1, dt, reuse_field=True)
        mprof = ctx.profile(reset=True)
        ctx.set_profiling(False)
        mstages = {k: {"launches": v["launches"], "ms": round(v["ms"], 3),
                       "GB/s": round(v["bytes"] / (v["ms"] * 1e6), 1) if v["ms"] > 0 else None}
                   for k, v in mprof["stages"].items() if v["launches"]}
        mfs = mprof["fine_smooth"]
        mfine = ({"kernel": "k_gsrb_f4 (finest-level FP32 red-black half sweep)",
                  "launches": mfs["launches"], "avg_launch_ms": mfs["ms"] / mfs["launches"],
                  "algorithmic_bytes_per_launch": mfs["bytes"] / mfs["launches"],
                  "achieved_GBs": round(mfs["bytes"] / (mfs["ms"] * 1e6), 1)}
                 if mfs["launches"] else None)
        # force error of one mixed step against one FP64 step from the same state
        pos_m, vel_m = bm.download()
        box.upload(pos_m, vel_m, ic.mass)
        bm.upload(pos_m, vel_m, ic.mass)
        a0, a1, dt = sched[W + K - 1]
        box.step(a0, a1, dt)
        bm.step(a0, a1, dt)
        g64, gmx = box.grav_vector(), bm.grav_vector()
        p64, v64 = box.download()
        pmx, vmx = bm.download()
        dpos = (pmx - p64 + 0.5) % 1.0 - 0.5
        line["mixed_reuse"] = {
            "value": allreduce_sum(ws, float(npart) * K, torch.device("cuda", local)) / (ms_m / 1e3),
            "ms_per_step": ms_m / K,
            "speedup_vs_plain_fp64_same_schedule": ms_r / ms_m,
            "speedup_vs_plain_fp64_reference_schedule": ms_max / ms_m,
            "outer_iters_mean": float(np.mean([m["vcycles"] for m in minfo])),
            "inner_vcycles_mean": float(np.mean([m["inner_vcycles"] for m in minfo])),
            "force_rel_l2_vs_fp64": rel_l2(gmx, g64),
            "vel_rel_l2_vs_fp64": float(np.linalg.norm(vmx - v64) / np.linalg.norm(v64)),
            "pos_err_cells_rms": float(np.sqrt(np.mean(dpos ** 2))) * n,
            "stages": mstages, "fine_smooth": mfine,
            "note": "same schedule: against reuse_field (the FP64 form, one solve per step); "
                    "errors: one step from the same state at the last timed a (the FP64 form "
                    "equals the FP64 oracle bitwise in the parity tests); stages: CUDA events "
                    "of 3 further steps outside the timed region"}
        # the mixed form on the headline's own schedule (two deposits + solves per step),
        # the same W + K steps from the same ICs
        bm.upload(ic.pos, ic.vel, ic.mass)
        for a0, a1, dt in sched[:W]:
            bm.step(a0, a1, dt)
        torch.cuda.synchronize()
        e0.record(stream)
        for a0, a1, dt in sched[W:W + K]:
            bm.step(a0, a1, dt)
        e1.record(stream)
        torch.cuda.synchronize()
        ms_mr = allreduce_max(ws, e0.elapsed_time(e1), torch.device("cuda", local))
        pos_m, vel_m = bm.download()
        box.upload(pos_m, vel_m, ic.mass)
        bm.upload(pos_m, vel_m, ic.mass)
        a0, a1, dt = sched[W + K - 1]
        box.step(a0, a1, dt)
        bm.step(a0, a1, dt)
        line["mixed_reference_schedule"] = {
            "value": allreduce_sum(ws, float(npart) * K, torch.device("cuda", local)) / (ms_mr / 1e3),
            "unit": UNIT, "ms_per_step": ms_mr / K,
            "speedup_vs_plain_fp64_same_schedule": ms_max / ms_mr,
            "force_rel_l2_vs_fp64": rel_l2(bm.grav_vector(), box.grav_vector()),
            "note": "the headline's workload and schedule (old- and new-time deposit + solve per "
                    "step) in the mixed form; the ratio is against the headline value; force error: "
                    "one step from the same state at the last timed a"}
        bm.close()

    # ---- end to end through the C ABI with pinned host buffers ----
    if not args.no_e2e:
        hpos = torch.empty((npart, 3), dtype=torch.float64, pin_memory=True)
        hvel = torch.empty((npart, 3), dtype=torch.float64, pin_memory=True)
        hpos.numpy()[:] = ic.pos
        hvel.numpy()[:] = ic.vel
        for a0, a1, dt in sched[:W]:
            box.step_host_ptr(hpos.data_ptr(), hvel.data_ptr(), ic.mass, a0, a1, dt)
        barrier(ws)
        torch.cuda.synchronize()
        t0 = time.perf_counter()
        e0.record(stream)
        vc_e = []
        for a0, a1, dt in sched[W:W + K]:
            inf = box.step_host_ptr(hpos.data_ptr(), hvel.data_ptr(), ic.mass, a0, a1, dt)
            vc_e.append((inf["old_solve"]["vcycles"], inf["new_solve"]["vcycles"]))
        e1.record(stream)
        torch.cuda.synchronize()
        wall = time.perf_counter() - t0
        barrier(ws)
        ms_e = allreduce_max(ws, e0.elapsed_time(e1), torch.device("cuda", local))
        line["e2e"] = {"value": allreduce_sum(ws, float(npart) * K, torch.device("cuda", local))
                       / (ms_e / 1e3), "unit": UNIT,
                       "h2d_bytes_per_step": int(hpos.numel() * 8 + hvel.numel() * 8),
                       "d2h_bytes_per_step": int(hpos.numel() * 8 + hvel.numel() * 8),
                       "ms_per_step": ms_e / K, "wall_ms_per_step": 1e3 * wall / K,
                       "vcycles_per_step": {"old_mean": float(np.mean([v[0] for v in vc_e])),
                                            "new_mean": float(np.mean([v[1] for v in vc_e]))},
                       "api": "nyxpm_step_host per step (upload + step + download in one call; "
                              "the transfers overlap the step on a second stream; pinned host "
                              "buffers)"}
        # the same through the mixed form (FP32 on the device, FP64 host buffers)
        bm = Box(ctx, n, 1.0, npart, precision="mixed")
        hpos.numpy()[:] = ic.pos
        hvel.numpy()[:] = ic.vel
        for a0, a1, dt in sched[:W]:
            bm.step_host_ptr(hpos.data_ptr(), hvel.data_ptr(), ic.mass, a0, a1, dt)
        barrier(ws)
        torch.cuda.synchronize()
        t0 = time.perf_counter()
        e0.record(stream)
        for a0, a1, dt in sched[W:W + K]:
            bm.step_host_ptr(hpos.data_ptr(), hvel.data_ptr(), ic.mass, a0, a1, dt)
        e1.record(stream)
        torch.cuda.synchronize()
        wall_m = time.perf_counter() - t0
        barrier(ws)
        ms_em = allreduce_max(ws, e0.elapsed_time(e1), torch.device("cuda", local))
        bm.close()
        line["mixed_e2e"] = {
            "value": allreduce_sum(ws, float(npart) * K, torch.device("cuda", local)) / (ms_em / 1e3),
            "unit": UNIT, "h2d_bytes_per_step": int(hpos.numel() * 8 + hvel.numel() * 8),
            "d2h_bytes_per_step": int(hpos.numel() * 8 + hvel.numel() * 8),
            "ms_per_step": ms_em / K, "wall_ms_per_step": 1e3 * wall_m / K,
            "speedup_vs_fp64_e2e": ms_e / ms_em,
            "api": "nyxpm_step_host on a mixed box (the headline's schedule; FP64 host buffers in "
                   "and out, the transfers overlapped with the step on a second stream)"}

    # ---- batched ensemble and continuous-batching serving (rank 0, N = 1) ----
    tuning = None
    if rank == 0 and ws == 1 and not args.no_ensemble:
        line["ensemble"] = run_ensemble_form(
            ctx, args.ensemble_boxes, args.ensemble_steps,
            [int(v) for v in args.tuning.split(",")] if args.tuning else None, stream)
        tuning = line["ensemble"]["tuning"]
    if rank == 0 and ws == 1 and not args.no_serving:
        line["serving"] = run_serving_form(ctx, args.serving_requests, tuning)
    if rank == 0 and ws == 1 and not args.no_c3:
        box.close()
        box = None
        line["c3"] = run_c3_form(ctx, stream)
    if rank == 0 and ws == 1 and not args.no_amr:
        line["amr"] = run_amr_form(ctx, stream, n0=args.amr_n0)

    # ---- CPU baseline: the oracle on a bounded sample, rank 0 at N=1 ----
    if rank == 0 and ws == 1 and not args.no_cpu_baseline:
        # about 10 s of CPU work: the first steps of the schedule, at most 30 s
        done, secs, threads, _ = oracle_steps(ic, sched[:8], n, 30.0)
        line["cpu_baseline"] = {
            "value": npart * done / secs, "unit": UNIT, "cores": threads, "kind": "port",
            "seconds": secs,
            "sample": f"the first {done} FP64 PM steps of the {n}^3 workload from a=0.02 (reference "
                      f"schedule), C++/OpenMP oracle on {threads} host threads"}
    if box is not None:
        box.close()
    ctx.close()
    if rank == 0:
        print(json.dumps(line), flush=True)
    if ws > 1:
        import torch.distributed as dist
        dist.destroy_process_group()
    return 0


def run_accuracy(args):
    """Mixed-precision accuracy on the 512^3 configuration (P(k) ~ k^-2.5, seed 3,
    a 0.02 -> 0.5 in 50 equal-da steps, reference schedule).  The comparison is the
    FP64 form, which equals the FP64 oracle bit for bit in the parity tests (the
    512^3 first step included).  Two measures at each reported step k:
      * one step: both forms take step k from the same FP64 state (the FP64
        run's state after step k-1) -- the error one mixed step adds;
      * free running: both forms run from the ICs to step k on their own -- the
        accumulated difference of two trajectories of a chaotic system.
    Positions are compared as displacements from the unperturbed lattice
    (minimum image), so the lattice offset does not hide the error."""
    import numpy as np
    import torch
    from nyx_gb300 import _lib
    _lib.load()
    from nyx_gb300.ics import zeldovich_ics
    from nyx_gb300.pm import Box, Context

    n, L = args.accuracy_n, 1.0
    report_at = sorted({int(s) for s in args.accuracy_steps.split(",")})
    nsteps = max(report_at)
    t0 = time.perf_counter()
    ic = zeldovich_ics(n, L, -2.5, 3, A_START, rms_disp_cells=0.2)
    t_ic = time.perf_counter() - t0
    npart = len(ic.pos)
    ctx = Context(device=0, mg_fused_edge=args.fused_edge)
    sched = ctx.step_schedule(A_START, A_END, NSTEPS_CFG)[:nsteps]

    def rel(a, b):
        return float(np.linalg.norm((a - b).ravel()) / np.linalg.norm(b.ravel()))

    def mr(f):
        return f - f.mean()

    def minimg(d):
        return (d + 0.5 * L) % L - 0.5 * L

    def compare(bm, bf):
        rho_m, rho_f = bm.deposit(), bf.deposit()
        out = {"rho": rel(rho_m, rho_f), "phi": rel(mr(bm.get_phi()), mr(bf.get_phi())),
               "g": rel(bm.grav_vector(), bf.grav_vector())}
        pm_, vm_ = bm.download()
        pf_, vf_ = bf.download()
        disp = minimg(pf_ - ic.lattice)
        out["x"] = float(np.linalg.norm(minimg(pm_ - pf_)) / np.linalg.norm(disp))
        out["v"] = rel(vm_, vf_)
        out["x_err_cells_max"] = float(np.abs(minimg(pm_ - pf_)).max() * n / L)
        return out

    free_f = Box(ctx, n, L, npart)
    free_m = Box(ctx, n, L, npart, precision="mixed")
    one_f = Box(ctx, n, L, npart)
    one_m = Box(ctx, n, L, npart, precision="mixed")
    for b in (free_f, free_m):
        b.upload(ic.pos, ic.vel, ic.mass)
    rows = []
    vcyc = []
    for k, (a0, a1, dt) in enumerate(sched, start=1):
        if k in report_at:
            pos, vel = free_f.download()
            for b in (one_f, one_m):
                b.upload(pos, vel, ic.mass)
            one_f.step(a0, a1, dt)
            mi = one_m.step(a0, a1, dt)
            row = {"step": k, "a": a1, "one_step": compare(one_m, one_f)}
            row["mixed_outer_iters"] = mi["new_solve"]["vcycles"]
            row["mixed_inner_vcycles"] = mi["new_solve"]["inner_vcycles"]
        fi = free_f.step(a0, a1, dt)
        free_m.step(a0, a1, dt)
        vcyc.append(fi["new_solve"]["vcycles"])
        if k in report_at:
            row["free_running"] = compare(free_m, free_f)
            row["fp64_vcycles"] = fi["new_solve"]["vcycles"]
            rows.append(row)
            print(json.dumps(row), file=sys.stderr, flush=True)
    for b in (free_f, free_m, one_f, one_m):
        b.close()
    ctx.close()
    line = {"report": "mixed-precision accuracy vs FP64", "n_grid": n, "n_particles": npart,
            "workload": f"{n}^3 particles on a {n}^3 periodic grid, Zel'dovich ICs P(k)~k^-2.5 "
                        f"seed 3, a {A_START}->{A_END} in {NSTEPS_CFG} equal-da steps, reference "
                        f"schedule, MG rel tol 1e-10",
            "target": "force (g) relative L2 <= 1e-6", "rows": rows,
            "ic_seconds": t_ic, "seconds": time.perf_counter() - t0}
    print(json.dumps(line), flush=True)
    return 0


def run_ensemble_only(args):
    import torch
    from nyx_gb300 import _lib
    _lib.load()
    from nyx_gb300.pm import Context
    ctx = Context(device=0, mg_fused_edge=args.fused_edge)
    stream = torch.cuda.ExternalStream(ctx.stream, device=torch.device("cuda", 0))
    fixed = [int(v) for v in args.tuning.split(",")] if args.tuning else None
    out = run_ensemble_form(ctx, args.ensemble_boxes, args.ensemble_steps, fixed, stream)
    ctx.close()
    print(json.dumps({"ensemble": out}), flush=True)
    return 0


def main():
    args = parse()
    if args.accuracy:
        return run_accuracy(args)
    if args.ensemble_only:
        return run_ensemble_only(args)
    if args.amr_only:
        return run_amr_only(args)
    if args.impl == "reference":
        return run_reference(args)
    return run_ours(args)


if __name__ == "__main__":
    sys.exit(main())
