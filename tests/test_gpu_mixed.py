"""GPU accuracy of the mixed-precision form (FP32 cell-relative particles, FP32
deposit and V-cycles inside FP64 defect correction) against the FP64 oracle.

Tolerance: relative L2 <= 1e-6 for the force (gravity vector) and for phi,
density and particle state, per step from identical input state; the FP64
residual of the defect-corrected solve meets the same 1e-10 relative
tolerance as the FP64 form.
"""
from __future__ import annotations

import numpy as np
import pytest

from nyx_gb300.pm import Box
from oracle import oracle as O
from tests.pm_cases import (config1_ics, equal_da_schedule, mean_removed, min_image, rel_l2,
                            true_resnorm)

pytestmark = pytest.mark.gpu

TOL = 1e-6


def displacement_err(gpos, opos, lattice, L):
    d = min_image(gpos - opos, L)
    disp = min_image(opos - lattice, L)
    return float(np.linalg.norm(d) / np.linalg.norm(disp))


@pytest.mark.parametrize("reuse,n", [(False, 64), (True, 64), (False, 10)])
def test_mixed_step_by_step_vs_oracle(ctx, reuse, n):
    """n = 10 has rows of 5 compact cells: the one-cell-per-thread residual kernels."""
    L = 1.0
    ic = config1_ics(n, seed=1)
    p = O.Particles(ic.pos, ic.vel, ic.mass)
    pm = O.PMOracle(n, L, p, reuse_field=reuse)
    b = Box(ctx, n, L, p.np, precision="mixed")
    if reuse:
        pm.init_field(0.02)
    for a0, a1, dt in equal_da_schedule(0.02, 0.05, 4):
        pos, vel = p.by_id()
        b.upload(pos, vel, ic.mass)
        if reuse:
            b.set_phi(pm.phi)
        info = b.step(a0, a1, dt, reuse_field=reuse)
        pm.step(a0, a1, dt)
        new = info["new_solve"]
        assert new["resnorm"] <= 1e-10 * max(new["bnorm"], new["resnorm0"]) * (1 + 1e-9)
        assert new["inner_vcycles"] >= new["vcycles"]
        # the residual of the returned phi, recomputed in FP64 by the oracle
        r_true, bnorm = true_resnorm(b, n, L, a1)
        assert r_true <= 1.05e-10 * max(bnorm, new["resnorm0"]), (r_true, bnorm)
        e_rho = rel_l2(b.deposit(), pm.rho)
        e_phi = rel_l2(mean_removed(b.get_phi()), mean_removed(pm.phi))
        e_g = rel_l2(b.grav_vector(), pm.g)
        gpos, gvel = b.download()
        opos, ovel = p.by_id()
        e_x = displacement_err(gpos, opos, ic.lattice, L)
        e_v = rel_l2(gvel, ovel)
        assert max(e_rho, e_phi, e_g, e_x, e_v) <= TOL, (e_rho, e_phi, e_g, e_x, e_v)


def test_mixed_free_running_config1(ctx):
    """10 steps a 0.02 -> 0.05 without resetting to the oracle: errors stay small."""
    n, L = 64, 1.0
    ic = config1_ics(n, seed=1)
    sched = ctx.step_schedule(0.02, 0.05, 10)
    b = Box(ctx, n, L, len(ic.pos), precision="mixed")
    b.upload(ic.pos, ic.vel, ic.mass)
    for a0, a1, dt in sched:
        b.step(a0, a1, dt)
    gpos, gvel = b.download()
    p = O.Particles(ic.pos, ic.vel, ic.mass)
    pm = O.PMOracle(n, L, p)
    for a0, a1, dt in sched:
        pm.step(a0, a1, dt)
    opos, ovel = p.by_id()
    assert displacement_err(gpos, opos, ic.lattice, L) <= 1e-5
    assert rel_l2(gvel, ovel) <= 1e-5
    assert rel_l2(b.grav_vector(), pm.g) <= 1e-5


@pytest.mark.parametrize("n", [6, 48])
def test_mixed_small_and_odd_grids(ctx, n):
    from nyx_gb300.ics import zeldovich_ics
    ic = zeldovich_ics(n, 2.0, -2.0, n + 1, 0.05, rms_disp_cells=0.3)
    p = O.Particles(ic.pos, ic.vel, ic.mass)
    pm = O.PMOracle(n, 2.0, p)
    b = Box(ctx, n, 2.0, len(ic.pos), precision="mixed")
    b.upload(ic.pos, ic.vel, ic.mass)
    (a0, a1, dt), = equal_da_schedule(0.05, 0.06, 1)
    b.step(a0, a1, dt)
    pm.step(a0, a1, dt)
    assert rel_l2(b.grav_vector(), pm.g) <= TOL
    gpos, gvel = b.download()
    opos, ovel = p.by_id()
    assert rel_l2(gvel, ovel) <= TOL


def test_mixed_deposit_conserves_mass_and_is_deterministic(ctx):
    n = 128
    from nyx_gb300.ics import zeldovich_ics
    ic = zeldovich_ics(n, 1.0, -2.5, 9, 0.02)
    b = Box(ctx, n, 1.0, len(ic.pos), precision="mixed")
    b.upload(ic.pos, ic.vel, ic.mass)
    r1 = b.deposit()
    b.redistribute()
    r2 = b.deposit()
    assert np.array_equal(r1, r2)
    assert r1.sum() * (1.0 / n) ** 3 == pytest.approx(ic.mass * len(ic.pos), rel=1e-5)


def test_mixed_drift_rebinning_at_cell_origin(ctx):
    """A particle at a cell origin drifting back by a sub-ulp distance stays at
    (almost) the same position: its FP32 offset rounds up to 1 and must move it
    to the next cell's origin, not one cell back."""
    n, L = 16, 1.0
    idx = np.arange(n)
    Z, Y, X = np.meshgrid(idx, idx, idx, indexing="ij")
    pos = np.stack([X.ravel(), Y.ravel(), Z.ravel()], 1) * (L / n)   # cell origins: offset 0
    vel = np.zeros_like(pos)
    b = Box(ctx, n, L, len(pos), precision="mixed")
    mass = 1e9
    a, dt = 0.5, 1e-6
    # drift in cells = dt / a * v / dx = -1e-9
    vel[:, 0] = -1e-9 * a * (L / n) / dt
    b.upload(pos, vel, mass)
    b.init_field(a)                        # uniform lattice: g = 0
    assert np.abs(b.grav_vector()).max() < 1e-6 * mass
    b.kick_drift(dt, a, a)
    gpos, _ = b.download()
    err = np.abs(min_image(gpos - pos, L)).max() / (L / n)
    assert err < 1e-6, err


@pytest.mark.parametrize("n", [64, 48])
def test_mixed_zero_guess_solve_meets_the_fp64_tolerance(ctx, n):
    """A zero-guess solve (its first correction is as large as phi, so the error
    bound forces one FP64 recomputation of the residual): the residual of the
    returned phi, recomputed by the oracle in FP64, meets the tolerance."""
    L = 1.0
    ic = config1_ics(n, seed=4)
    b = Box(ctx, n, L, len(ic.pos), precision="mixed")
    b.upload(ic.pos, ic.vel, ic.mass)
    b.deposit(read_back=False)
    info = b.solve_phi(0.05, zero_guess=True)
    r_true, bnorm = true_resnorm(b, n, L, 0.05)
    assert info["resnorm"] <= 1e-10 * max(info["bnorm"], info["resnorm0"]) * (1 + 1e-9)
    assert r_true <= 1.05e-10 * max(bnorm, info["resnorm0"]), (r_true, bnorm, info)
    # a second solve from that phi (no zero guess) stays within the tolerance too
    info2 = b.solve_phi(0.05)
    r2, _ = true_resnorm(b, n, L, 0.05)
    assert r2 <= 1.05e-10 * max(bnorm, info2["resnorm0"]), (r2, info2)
    b.close()


def test_mixed_deposit_clustered_vs_oracle(ctx):
    """The FP32 deposit on clustered particles: windows of a tile holding many
    chunks of particles, keys of up to a warp's worth (summed in order by one
    thread) and keys longer than a warp (summed by the warp pass), against the
    FP64 oracle's density; deterministic run to run."""
    n, L = 32, 1.0
    rng = np.random.default_rng(21)
    pos = np.concatenate([rng.random((20000, 3)),                      # background
                          0.40 + 0.03 * rng.random((6000, 3)),         # keys of ~5-40
                          0.71 + 0.004 * rng.random((1500, 3)),        # keys of hundreds
                          0.1 + 0.5 * rng.random((4000, 3)) * [1, 0.05, 0.05]])
    mass = 3.0e9
    p = O.Particles(pos, np.zeros_like(pos), mass)
    rho_o = O.deposit(n, L, p, O.sort(n, L, p))
    b = Box(ctx, n, L, len(pos), precision="mixed")
    b.upload(pos, np.zeros_like(pos), mass)
    r1 = b.deposit()
    b.redistribute()
    r2 = b.deposit()
    assert np.array_equal(r1, r2)
    assert rel_l2(r1, rho_o) <= 2e-6, rel_l2(r1, rho_o)
    big = rho_o > 0.1 * rho_o.max()
    assert np.abs(r1[big] / rho_o[big] - 1).max() <= 1e-5
    b.close()
