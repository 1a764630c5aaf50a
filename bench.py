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
    ap.add_argument("--quick", action="store_true",
                    help="headline timing only (no reuse-field pass, e2e or CPU baseline); "
                         "the command the ncu captures run")
    a = ap.parse_args()
    if a.quick:
        a.no_cpu_baseline = a.no_e2e = a.no_reuse = True
    else:
        a.no_reuse = False
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
    ic = zeldovich_ics(n, 1.0, -2.0, 2 + rank, A_START, rms_disp_cells=0.2)
    npart = len(ic.pos)
    ctx = Context(device=local)
    stream = torch.cuda.ExternalStream(ctx.stream, device=torch.device("cuda", local))
    sched = schedule(ctx, W + K)
    box = Box(ctx, n, 1.0, npart)
    box.upload(ic.pos, ic.vel, ic.mass)

    # ---- device-resident run: warm-up, then K timed steps ----
    for a0, a1, dt in sched[:W]:
        box.step(a0, a1, dt)
    ctx.set_profiling(True)
    ctx.profile(reset=True)
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
    prof = ctx.profile(reset=True)
    ctx.set_profiling(False)
    ms_max = allreduce_max(ws, ms, torch.device("cuda", local))
    total_units = allreduce_sum(ws, float(npart) * K, torch.device("cuda", local))
    value = total_units / (ms_max / 1e3)

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
        kname = "k_gsrb (finest-level red-black half sweep)"
        tr = traffic.get("k_gsrb_fine")
    else:
        st = stages[dom]
        per_launch = st["bytes"] / max(st["launches"], 1)
        avg_ms = st["ms"] / max(st["launches"], 1)
        kname = dom
        tr = traffic.get(dom)
    achieved = per_launch / (avg_ms * 1e6)
    roofline = {"bound": "hbm", "kernel": kname, "achieved": round(achieved, 1),
                "peak": peak, "peak_source": peak_kind, "unit": "GB/s",
                "frac": round(achieved / peak, 4),
                "traffic": (tr * (n / traffic.get("n", n)) ** 3 if tr else None),
                "algorithmic_bytes_per_launch": per_launch, "avg_launch_ms": avg_ms,
                "dominant_stage_share": round(stages[dom]["ms"] / sum(v["ms"] for v in stages.values()), 3)}

    line = {
        "metric": METRIC, "value": value, "unit": UNIT, "n_gpus": ws, "steps": K, "warmup": W,
        "ms_per_step": ms_max / K, "higher_is_better": True, "scaling": "weak",
        "vs_baseline": None, "dtype": "f64", "data": "synthetic",
        "config": workload_config(n, W, K),
        "roofline": roofline, "clocks": clk, "gpu_launches": int(launches),
        "stages": stage_rows,
        "vcycles_per_step": {"old_mean": float(np.mean([v[0] for v in vcycles])),
                             "new_mean": float(np.mean([v[1] for v in vcycles]))},
    }

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
            "ms_per_step": ms_m / K, "speedup_vs_plain_fp64": ms_max / ms_m,
            "outer_iters_mean": float(np.mean([m["vcycles"] for m in minfo])),
            "inner_vcycles_mean": float(np.mean([m["inner_vcycles"] for m in minfo])),
            "force_rel_l2_vs_fp64": float(np.linalg.norm(gmx - g64) / np.linalg.norm(g64)),
            "vel_rel_l2_vs_fp64": float(np.linalg.norm(vmx - v64) / np.linalg.norm(v64)),
            "pos_err_cells_rms": float(np.sqrt(np.mean(dpos ** 2))) * n,
            "note": "one step from the same state at the last timed a; the FP64 form equals the "
                    "FP64 oracle bitwise in the parity tests"}
        bm.close()

    # ---- end to end through the C ABI with pinned host buffers ----
    if not args.no_e2e:
        hpos = torch.empty((npart, 3), dtype=torch.float64, pin_memory=True)
        hvel = torch.empty((npart, 3), dtype=torch.float64, pin_memory=True)
        hpos.numpy()[:] = ic.pos
        hvel.numpy()[:] = ic.vel
        for a0, a1, dt in sched[:W]:
            box.upload_ptr(hpos.data_ptr(), hvel.data_ptr(), ic.mass)
            box.step(a0, a1, dt)
            box.download_ptr(hpos.data_ptr(), hvel.data_ptr())
        barrier(ws)
        torch.cuda.synchronize()
        t0 = time.perf_counter()
        e0.record(stream)
        for a0, a1, dt in sched[W:W + K]:
            box.upload_ptr(hpos.data_ptr(), hvel.data_ptr(), ic.mass)
            box.step(a0, a1, dt)
            box.download_ptr(hpos.data_ptr(), hvel.data_ptr())
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
                       "api": "nyxpm_box_upload + nyxpm_step + nyxpm_box_download per step"}

    # ---- CPU baseline: the oracle on a bounded sample, rank 0 at N=1 ----
    if rank == 0 and ws == 1 and not args.no_cpu_baseline:
        done, secs, threads, _ = oracle_steps(ic, sched[:1], n, 30.0)
        line["cpu_baseline"] = {
            "value": npart * done / secs, "unit": UNIT, "cores": threads, "kind": "port",
            "sample": f"{done} FP64 PM step(s) of the {n}^3 workload from a=0.02 (reference "
                      f"schedule), C++/OpenMP oracle on {threads} host threads"}
    box.close()
    ctx.close()
    if rank == 0:
        print(json.dumps(line), flush=True)
    if ws > 1:
        import torch.distributed as dist
        dist.destroy_process_group()
    return 0


def main():
    args = parse()
    if args.impl == "reference":
        return run_reference(args)
    return run_ours(args)


if __name__ == "__main__":
    sys.exit(main())
