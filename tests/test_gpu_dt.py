"""GPU time-step control against the oracle, through the C ABI.

* the particle time-step limit (NyxParticleContainer::estTimestep) is a GPU
  reduction over particles; on the FP64 form it equals the oracle's bit for bit
  (minimum of IEEE-rounded quotients and square roots, order-independent);
* computeNewDt chains it with the host a-change limit, change_max and
  stop_time; a CFL-limited run (dt chosen every step) follows the oracle's
  run step for step;
* the mixed form's limit agrees to relative 1e-6.
"""
from __future__ import annotations

import numpy as np
import pytest

from nyx_gb300.pm import Box
from oracle import oracle as O
from tests.pm_cases import config1_ics, rel_l2

pytestmark = pytest.mark.gpu

OMM, OMR, H = 1.0, 0.0, 0.675


def oracle_new_dt(n, L, p, g, a, time, dt_old, cfl=0.5, change_max=1.1, stop_time=-1.0, **kw):
    est = 1e200
    part = O.est_time_step(n, L, p, g, cfl, a)
    if part > 0:
        est = min(est, part)
    est, st = O.comoving_est_dt(OMM, OMR, H, a, est, **kw)
    assert st == 0
    if dt_old > 0:
        est = min(est, change_max * dt_old)
    if stop_time >= 0 and time + est > stop_time - 0.001 * est:
        est = stop_time - time
    return est, O.integrate_a(OMM, OMR, H, a, est)


def test_particle_limit_equals_oracle(ctx):
    n, L, a = 64, 1.0, 0.02
    ic = config1_ics(n, seed=1)
    b = Box(ctx, n, L, len(ic.pos))
    b.upload(ic.pos, ic.vel, ic.mass)
    b.init_field(a)
    p = O.Particles(ic.pos, ic.vel, ic.mass)
    pm = O.PMOracle(n, L, p)
    pm.init_field(a)
    for cfl in (0.5, 0.1):
        assert b.est_time_step(cfl, a) == O.est_time_step(n, L, p, pm.g, cfl, a)
    # after a step: new positions, velocities and field
    a1 = ctx.integrate_comoving_a(a, 2e-6)
    b.step(a, a1, 2e-6)
    pm.step(a, a1, 2e-6)
    assert b.est_time_step(0.5, a1) == O.est_time_step(n, L, pm.p, pm.g, 0.5, a1)
    b.close()


def test_cfl_limited_run_follows_oracle(ctx):
    """Six steps with dt = computeNewDt every step (particle CFL, 1% a-change,
    change_max) on the GPU and in the oracle, from the same ICs."""
    n, L = 32, 1.0
    ic = config1_ics(n, seed=3, a_init=0.05)
    b = Box(ctx, n, L, len(ic.pos))
    b.upload(ic.pos, ic.vel, ic.mass)
    p = O.Particles(ic.pos, ic.vel, ic.mass)
    pm = O.PMOracle(n, L, p)
    a = 0.05
    b.init_field(a)
    pm.init_field(a)
    t, dt_old = 0.0, -1.0
    for _ in range(6):
        dt, a_new = b.compute_new_dt(t, a, dt_old, cfl=0.5)
        want_dt, want_a = oracle_new_dt(n, L, pm.p, pm.g, a, t, dt_old)
        assert (dt, a_new) == (want_dt, want_a)
        b.step(a, a_new, dt)
        pm.step(a, a_new, dt)
        t, a, dt_old = t + dt, a_new, dt
    gpos, gvel = b.download()
    opos, ovel = pm.p.by_id()
    assert rel_l2(gvel, ovel) <= 1e-12
    # stop_time clips the last step
    dt, _ = b.compute_new_dt(t, a, dt_old, stop_time=t + 1e-9)
    assert dt == pytest.approx(1e-9, rel=1e-6)
    b.close()


def test_mixed_particle_limit(ctx):
    n, L, a = 64, 1.0, 0.02
    ic = config1_ics(n, seed=1)
    b = Box(ctx, n, L, len(ic.pos), precision="mixed")
    b.upload(ic.pos, ic.vel, ic.mass)
    b.init_field(a)
    p = O.Particles(ic.pos, ic.vel, ic.mass)
    pm = O.PMOracle(n, L, p)
    pm.init_field(a)
    got, want = b.est_time_step(0.5, a), O.est_time_step(n, L, p, pm.g, 0.5, a)
    assert abs(got - want) <= 1e-6 * want
    b.close()


def test_no_field_is_an_error(ctx):
    from nyx_gb300.pm import NyxPMError
    ic = config1_ics(16, seed=1)
    b = Box(ctx, 16, 1.0, len(ic.pos))
    b.upload(ic.pos, ic.vel, ic.mass)
    with pytest.raises(NyxPMError):
        b.est_time_step(0.5, 0.02)
    b.close()
