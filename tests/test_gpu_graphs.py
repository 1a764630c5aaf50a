"""Solver iterations replayed from a per-box CUDA graph give the same results, bit
for bit, as the same launches enqueued one by one (the eager path, which runs
while per-launch profiling is on), for the FP64 and the mixed form.  The launch
count a replay reports equals the eager count.
"""
from __future__ import annotations

import numpy as np
import pytest

from nyx_gb300.pm import Box
from tests.pm_cases import config1_ics, equal_da_schedule

pytestmark = pytest.mark.gpu


def run(ctx, precision, profiling, n=32, steps=3):
    ic = config1_ics(n, seed=5)
    ctx.set_profiling(profiling)
    try:
        b = Box(ctx, n, 1.0, len(ic.pos), precision=precision)
        b.upload(ic.pos, ic.vel, ic.mass)
        infos = []
        l0 = ctx.launch_count()
        for a0, a1, dt in equal_da_schedule(0.02, 0.05, steps):
            infos.append(b.step(a0, a1, dt))
        launches = ctx.launch_count() - l0
        pos, vel = b.download()
        phi = b.get_phi()
        b.close()
    finally:
        ctx.profile(reset=True)
        ctx.set_profiling(False)
    return pos, vel, phi, infos, launches


@pytest.mark.parametrize("precision", ["fp64", "mixed"])
def test_graph_replay_equals_eager_launches(ctx, precision):
    pe, ve, fe, ie, le = run(ctx, precision, profiling=True)
    pg, vg, fg, ig, lg = run(ctx, precision, profiling=False)
    assert np.array_equal(pe, pg) and np.array_equal(ve, vg) and np.array_equal(fe, fg)
    assert ie == ig                      # the same iteration counts and norms
    assert le == lg
    assert all(i["new_solve"]["vcycles"] >= 1 for i in ig)


@pytest.mark.parametrize("n,edge", [(16, 16), (48, 16), (64, 16), (32, 32)])
def test_fused_coarse_vcycle_equals_one_launch_per_pass(ctx, n, edge):
    """mg_fused_edge = e cycles the levels of <= e cells per edge in one launch;
    0 launches every pass.  The mixed results are the same bits (n = 16: the
    whole V-cycle is fused; 48: levels 12, 6 and the 3^3 bottom, rows of odd
    length and non-power-of-two edges)."""
    from nyx_gb300.pm import Context
    assert ctx.params.mg_fused_edge == 16
    fused = Context(mg_fused_edge=edge)
    plain = Context(mg_fused_edge=0)
    try:
        a = run(fused, "mixed", profiling=False, n=n, steps=2)
        b = run(plain, "mixed", profiling=False, n=n, steps=2)
    finally:
        fused.close()
        plain.close()
    assert np.array_equal(a[0], b[0]) and np.array_equal(a[1], b[1]) and np.array_equal(a[2], b[2])
    assert a[3] == b[3]
    assert a[4] < b[4]                   # fewer launches


@pytest.mark.parametrize("n", [32, 48, 64])
def test_fused_fp64_coarse_vcycle_equals_one_launch_per_pass(ctx, n):
    """The FP64 form fuses the levels of at most mg_fused_edge / 2 cells per edge
    below the finest (8^3 and 4^3 at the default; n = 48: 6^3 and the 3^3
    bottom).  Same bits as one launch per pass."""
    from nyx_gb300.pm import Context
    plain = Context(mg_fused_edge=0)
    try:
        a = run(ctx, "fp64", profiling=False, n=n, steps=2)
        b = run(plain, "fp64", profiling=False, n=n, steps=2)
    finally:
        plain.close()
    assert np.array_equal(a[0], b[0]) and np.array_equal(a[1], b[1]) and np.array_equal(a[2], b[2])
    assert a[3] == b[3]
    assert a[4] < b[4]
