"""GPU tests of the batched ensemble (mixed precision, one persistent launch per
stage over all boxes, captured step graphs).

* every box of an ensemble tracks the FP64 oracle run on its own
  (old-time field reused): after several steps the force (gravity vector) to
  <= 1e-6 relative L2 and particle state to <= 1e-5, on boxes of every size the
  ensemble configuration draws (32 .. 128 cells, one and half a particle per
  cell);
* a box's result is bitwise the same alone and inside a mix of other boxes;
* the deposit tile, sort bucket and smoother row shapes do not change results;
* the memory budget is enforced and freed memory is reused.
"""
from __future__ import annotations

import numpy as np
import pytest

from nyx_gb300.ensemble import BoxSpec, Ensemble, box_ics
from oracle import oracle as O
from tests.pm_cases import equal_da_schedule, min_image, rel_l2

pytestmark = pytest.mark.gpu


def run_ensemble(ctx, specs, ics, sched, tuning=None):
    arena = int(sum(Ensemble.box_bytes(s.n, s.np) for s in specs) * 1.3) + (64 << 20)
    ens = Ensemble(ctx, arena)
    if tuning:
        ens.set_tuning(**tuning)
    slots = []
    for s, ic in zip(specs, ics):
        slot = ens.add(s.n, s.L, s.np)
        ens.upload(slot, ic.pos, ic.vel, ic.mass)
        slots.append(slot)
    infos = []
    for a0, a1, dt in sched:
        infos.append(ens.step({s: a0 for s in slots}, {s: a1 for s in slots}, {s: dt for s in slots}))
    out = [ens.download(s) for s in slots]
    g = [ens.grav_vector(s) for s in slots]
    ens.close()
    return out, g, infos


SPECS = [BoxSpec(32, 1.0, 11, -2.0), BoxSpec(48, 0.5, 12, -1.6), BoxSpec(16, 1.0, 13, -2.4),
         BoxSpec(64, 0.5, 14, -2.2)]


# the sizes and particle fractions of the ensemble configuration's draws
ORACLE_SPECS = SPECS + [BoxSpec(96, 0.5, 15, -1.8), BoxSpec(128, 1.0, 16, -2.5),
                        BoxSpec(128, 0.5, 17, -1.5), BoxSpec(32, 0.5, 18, -2.1)]


def test_ensemble_matches_oracle_per_box(ctx):
    ics = [box_ics(s, 0.05) for s in ORACLE_SPECS]
    sched = equal_da_schedule(0.05, 0.08, 4)
    out, g, infos = run_ensemble(ctx, ORACLE_SPECS, ics, sched)
    assert all(i["boxes"] == len(ORACLE_SPECS) for i in infos)
    for s, ic, (pos, vel), gg in zip(ORACLE_SPECS, ics, out, g):
        p = O.Particles(ic.pos, ic.vel, ic.mass)
        pm = O.PMOracle(s.n, s.L, p, reuse_field=True)
        pm.init_field(0.05)
        for a0, a1, dt in sched:
            pm.step(a0, a1, dt)
        opos, ovel = p.by_id()
        disp = min_image(opos - ic.lattice, s.L)
        ex = np.linalg.norm(min_image(pos - opos, s.L)) / np.linalg.norm(disp)
        ev = rel_l2(vel, ovel)
        eg = rel_l2(gg, pm.g)
        assert eg <= 1e-6 and max(ex, ev) <= 1e-5, (s, ex, ev, eg)


def test_alone_equals_in_mix(ctx):
    ics = [box_ics(s, 0.05) for s in SPECS]
    sched = equal_da_schedule(0.05, 0.07, 3)
    mix, gmix, _ = run_ensemble(ctx, SPECS, ics, sched)
    for i in (0, 2):
        alone, galone, _ = run_ensemble(ctx, [SPECS[i]], [ics[i]], sched)
        assert np.array_equal(alone[0][0], mix[i][0]) and np.array_equal(alone[0][1], mix[i][1])
        assert np.array_equal(galone[0], gmix[i])


def test_shapes_do_not_change_results(ctx):
    ics = [box_ics(s, 0.05) for s in SPECS[:2]]
    sched = equal_da_schedule(0.05, 0.06, 2)
    base, _, _ = run_ensemble(ctx, SPECS[:2], ics, sched)
    for tuning in ({"deposit_tile": 1, "smooth_rows": 2, "sort_bucket": 512, "prolong_quad": 0},
                   {"deposit_tile": 2, "smooth_rows": 4, "sort_bucket": 1024}):
        other, _, _ = run_ensemble(ctx, SPECS[:2], ics, sched, tuning)
        for (p0, v0), (p1, v1) in zip(base, other):
            assert np.array_equal(p0, p1) and np.array_equal(v0, v1)


def test_one_graph_step_loops_on_the_device(ctx):
    """With max_outer = 1 every box needs more defect-correction iterations than
    the graph's fixed ones: the step graph's WHILE node runs them on the device,
    one graph launch per step, and the result equals the eager step's (profiling
    mode: the same kernels launched one by one, the extra iterations driven by the
    host), bit for bit."""
    ics = [box_ics(s, 0.05) for s in SPECS]
    sched = equal_da_schedule(0.05, 0.07, 3)
    graph, g_graph, infos = run_ensemble(ctx, SPECS, ics, sched, {"max_outer": 1})
    assert all(i["fallback_iters"] > 0 for i in infos), infos
    ctx.set_profiling(True)
    try:
        eager, g_eager, infos_e = run_ensemble(ctx, SPECS, ics, sched, {"max_outer": 1})
    finally:
        ctx.set_profiling(False)
        ctx.profile(reset=True)
    assert [i["fallback_iters"] for i in infos] == [i["fallback_iters"] for i in infos_e]
    for (p0, v0), (p1, v1), ga, gb in zip(graph, eager, g_graph, g_eager):
        assert np.array_equal(p0, p1) and np.array_equal(v0, v1) and np.array_equal(ga, gb)


def test_budget_and_reuse(ctx):
    one = Ensemble.box_bytes(32, 32 ** 3)
    ens = Ensemble(ctx, int(one * 2.2))
    a = ens.try_add(32, 1.0, 32 ** 3)
    b = ens.try_add(32, 1.0, 32 ** 3)
    assert a is not None and b is not None
    assert ens.try_add(32, 1.0, 32 ** 3) is None      # over budget
    ens.remove(a)
    c = ens.try_add(32, 1.0, 32 ** 3)
    assert c is not None
    with pytest.raises(Exception):
        ens.add(18, 1.0, 100)                          # 18 = 9 * 2 is not supported
    ens.close()


def test_profiled_eager_step_equals_graph_step(ctx):
    """With profiling on, the ensemble step runs its launches eagerly with stage
    events instead of replaying the captured graphs; the results are the same."""
    ics = [box_ics(s, 0.05) for s in SPECS[:3]]
    sched = equal_da_schedule(0.05, 0.07, 3)
    graphs, g0, _ = run_ensemble(ctx, SPECS[:3], ics, sched)
    ctx.set_profiling(True)
    ctx.profile(reset=True)
    try:
        eager, g1, _ = run_ensemble(ctx, SPECS[:3], ics, sched)
        prof = ctx.profile(reset=True)
    finally:
        ctx.set_profiling(False)
    for (p0, v0), (p1, v1), a, b in zip(graphs, eager, g0, g1):
        assert np.array_equal(p0, p1) and np.array_equal(v0, v1) and np.array_equal(a, b)
    assert prof["stages"]["smooth"]["launches"] > 0 and prof["stages"]["deposit"]["ms"] > 0


def test_fused_coarse_vcycle_gives_the_same_bits(ctx):
    """The coarse levels (<= 16 cells per edge) of every box cycled by one CTA per
    box (e_tail) against one launch per pass over all boxes: the same bits."""
    from nyx_gb300.pm import Context
    ics = [box_ics(s, 0.05) for s in SPECS]
    sched = equal_da_schedule(0.05, 0.07, 2)
    plain = Context(mg_fused_edge=0)
    try:
        out_p, g_p, _ = run_ensemble(plain, SPECS, ics, sched)
    finally:
        plain.close()
    out_f, g_f, _ = run_ensemble(ctx, SPECS, ics, sched)
    for (p0, v0), (p1, v1), a, b in zip(out_p, out_f, g_p, g_f):
        assert np.array_equal(p0, p1) and np.array_equal(v0, v1) and np.array_equal(a, b)
