"""Continuous-batching server for PM runs on one GPU.

Requests (grid size, number of steps, IC seed and slope) arrive over time.  The
server keeps one mixed-precision ``Ensemble`` whose device arena is the HBM
budget: a request is admitted when its box fits in what the arena has free
(arrival order; a request that does not fit waits, later ones that fit may
pass it after ``max_skip`` ticks of waiting are exhausted), its particles and
multigrid hierarchy stay resident while it runs, every engine tick advances all
admitted runs by one step in one batched step (one persistent launch per stage,
one graph replay), and a finished run is downloaded and its memory returned to
the arena at once, so requests that arrive while others are on the GPU join as
memory frees up.

``serve_sequential`` is the comparison: the same stream served by the plain
FP64 drop-in one run at a time, in arrival order, on the same step schedule as
the server (the old-time field reused: one deposit and one solve per step) or,
with ``reuse_field=False``, on Nyx's own two-solve schedule.

Each run uses equal-delta-a steps from a = 0.02 with delta a = 0.009 (the
ensemble configuration's 0.02 -> 0.2 in 20 steps).
"""
from __future__ import annotations

import math
import time
from dataclasses import dataclass, field

import numpy as np

from .ensemble import BoxSpec, Ensemble
from .pm import Box, Context

A_START = 0.02
DA = 0.009
SIZES = (32, 48, 64, 96, 128, 192)
WEIGHTS = (0.30, 0.25, 0.20, 0.12, 0.08, 0.05)


@dataclass
class Request:
    rid: int
    arrival: float          # seconds after the stream starts
    n: int
    nsteps: int
    seed: int
    slope: float
    L: float = 1.0
    fraction: float = 1.0

    @property
    def np(self) -> int:
        return int(math.ceil(self.fraction * self.n ** 3))

    def spec(self) -> BoxSpec:
        return BoxSpec(self.n, self.fraction, self.seed, self.slope, self.L)


@dataclass
class Result:
    rid: int
    arrival: float
    start: float
    done: float
    pos: np.ndarray | None = None
    vel: np.ndarray | None = None
    g: np.ndarray | None = None          # the gravity vector the run ended with

    @property
    def latency(self) -> float:
        return self.done - self.arrival


def request_stream(nreq: int, rate: float, seed: int = 5, sizes=SIZES, weights=WEIGHTS,
                   steps=(10, 40)) -> list[Request]:
    """Poisson arrivals at `rate` per second; n by the given weights; steps uniform."""
    rng = np.random.default_rng(seed)
    t = 0.0
    out = []
    w = np.asarray(weights, dtype=np.float64)
    w = w / w.sum()
    for r in range(nreq):
        t += rng.exponential(1.0 / rate) if rate > 0 else 0.0
        n = int(rng.choice(sizes, p=w))
        out.append(Request(rid=r, arrival=t, n=n, nsteps=int(rng.integers(steps[0], steps[1] + 1)),
                           seed=int(rng.integers(1, 2 ** 31 - 1)),
                           slope=float(rng.uniform(-2.5, -1.5))))
    return out


def schedule(ctx: Context, nsteps: int):
    return ctx.step_schedule(A_START, A_START + DA * nsteps, nsteps)


@dataclass
class _Run:
    req: Request
    slot: int
    sched: list
    k: int = 0
    start: float = 0.0


@dataclass
class ServeStats:
    results: list = field(default_factory=list)
    wall: float = 0.0
    ticks: int = 0
    max_active: int = 0
    peak_arena_bytes: int = 0
    particle_steps: int = 0

    def summary(self) -> dict:
        lat = np.array([r.latency for r in self.results]) if self.results else np.zeros(1)
        span = (max(r.done for r in self.results) - min(r.arrival for r in self.results)
                if self.results else 0.0)
        return {"completed": len(self.results), "runs_per_s": len(self.results) / span if span else 0.0,
                "p50_latency_s": float(np.percentile(lat, 50)),
                "p99_latency_s": float(np.percentile(lat, 99)),
                "mean_latency_s": float(lat.mean()), "wall_s": self.wall, "ticks": self.ticks,
                "max_concurrent_runs": self.max_active, "peak_arena_GB": self.peak_arena_bytes / 1e9,
                "particle_steps_per_s": self.particle_steps / self.wall if self.wall else 0.0}


def _keeps(keep, rid: int) -> bool:
    """keep: False, True (every run) or a set of request ids."""
    return bool(keep) and (keep is True or rid in keep)


class ContinuousBatchingServer:
    """keep_results: False, True or a set of request ids whose final particle
    state and gravity vector are downloaded into their Result."""

    def __init__(self, ctx: Context, budget_bytes: int, ic_provider, tuning: dict | None = None,
                 keep_results=False, max_skip: int = 64):
        self.ctx = ctx
        self.ens = Ensemble(ctx, budget_bytes)
        if tuning:
            self.ens.set_tuning(**{k: v for k, v in tuning.items()
                                   if k in ("deposit_tile", "smooth_rows", "inner_vcycles", "max_outer",
                                            "sort_bucket", "prolong_quad")})
        self.ic_provider = ic_provider
        self.keep = keep_results
        self.max_skip = max_skip

    def serve(self, requests: list[Request], realtime: bool = True) -> ServeStats:
        """Serve the stream; with realtime=False every request is available at once."""
        st = ServeStats()
        pending = sorted(requests, key=lambda r: r.arrival)
        queue: list[Request] = []
        active: dict[int, _Run] = {}
        skipped: dict[int, int] = {}
        t0 = time.perf_counter()
        i = 0
        while i < len(pending) or queue or active:
            now = time.perf_counter() - t0
            while i < len(pending) and (not realtime or pending[i].arrival <= now):
                queue.append(pending[i])
                i += 1
            # admission by memory budget in arrival order; a request that does not fit
            # waits and later ones that fit pass it, until it has waited max_skip ticks
            for qi, r in enumerate(list(queue)):
                slot = self.ens.try_add(r.n, r.L, r.np)
                if slot is None:
                    skipped[r.rid] = skipped.get(r.rid, 0) + 1
                    if skipped[r.rid] > self.max_skip:
                        break
                    continue
                ic = self.ic_provider(r)
                self.ens.upload(slot, ic.pos, ic.vel, ic.mass)
                run = _Run(req=r, slot=slot, sched=schedule(self.ctx, r.nsteps),
                           start=time.perf_counter() - t0)
                active[slot] = run
                queue.remove(r)
            if not active:
                if i < len(pending) and realtime:
                    wait = pending[i].arrival - (time.perf_counter() - t0)
                    if wait > 0:
                        time.sleep(min(wait, 0.05))
                    continue
                if queue:
                    raise RuntimeError("a request does not fit in the memory budget on its own")
                continue
            st.max_active = max(st.max_active, len(active))
            st.peak_arena_bytes = max(st.peak_arena_bytes, self.ens.arena_used())
            a0 = {s: run.sched[run.k][0] for s, run in active.items()}
            a1 = {s: run.sched[run.k][1] for s, run in active.items()}
            dt = {s: run.sched[run.k][2] for s, run in active.items()}
            self.ens.step(a0, a1, dt)
            st.ticks += 1
            for s, run in list(active.items()):
                run.k += 1
                st.particle_steps += run.req.np
                if run.k == len(run.sched):
                    pos = vel = g = None
                    if _keeps(self.keep, run.req.rid):
                        pos, vel = self.ens.download(s)
                        g = self.ens.grav_vector(s)
                    self.ens.remove(s)
                    del active[s]
                    st.results.append(Result(run.req.rid, run.req.arrival if realtime else 0.0,
                                             run.start, time.perf_counter() - t0, pos, vel, g))
        st.wall = time.perf_counter() - t0
        return st

    def close(self):
        self.ens.close()


def serve_sequential(ctx: Context, requests: list[Request], ic_provider, realtime: bool = True,
                     max_requests: int | None = None, reuse_field: bool = True,
                     keep_results=False) -> ServeStats:
    """The same stream served by the plain FP64 drop-in, one run at a time.
    reuse_field: the server's schedule (post_init solve, then one deposit and one
    solve per step); False: the reference's two solves per step."""
    st = ServeStats()
    reqs = sorted(requests, key=lambda r: r.arrival)
    if max_requests is not None:
        reqs = reqs[:max_requests]
    t0 = time.perf_counter()
    for r in reqs:
        if realtime:
            wait = r.arrival - (time.perf_counter() - t0)
            if wait > 0:
                time.sleep(wait)
        start = time.perf_counter() - t0
        ic = ic_provider(r)
        box = Box(ctx, r.n, r.L, r.np)
        box.upload(ic.pos, ic.vel, ic.mass)
        sched = schedule(ctx, r.nsteps)
        if reuse_field:
            box.init_field(sched[0][0])
        for a0, a1, dt in sched:
            box.step(a0, a1, dt, reuse_field=reuse_field)
        pos, vel = box.download()
        g = box.grav_vector() if _keeps(keep_results, r.rid) else None
        if not _keeps(keep_results, r.rid):
            pos = vel = None
        box.close()
        st.particle_steps += r.np * r.nsteps
        st.results.append(Result(r.rid, r.arrival if realtime else 0.0, start, time.perf_counter() - t0,
                                 pos, vel, g))
        st.max_active = 1
    st.wall = time.perf_counter() - t0
    return st
