"""GPU parity of the FP64 drop-in against the CPU oracle, through the C ABI.

Tolerance (FP64 form): relative L2 <= 1e-12 for density, mean-removed phi,
gravity vector and particle state; the V-cycle counts must be equal.  The
density uses the same summation order as the oracle, so it is compared bitwise.
"""
from __future__ import annotations

import math

import numpy as np
import pytest

from nyx_gb300.pm import Box, NyxPMError
from nyx_gb300.ics import zeldovich_ics
from oracle import oracle as O
from tests.pm_cases import (config1_ics, equal_da_schedule, load_zeldovich, mean_removed,
                            min_image, rel_l2, zeldovich_errors, zeldovich_particles,
                            zeldovich_schedule)

pytestmark = pytest.mark.gpu

TOL = 1e-12
GG = None


def ggrav():
    return -4.0 * math.pi * O.gconst()


def make_box(ctx, n, L, pos, vel, mass):
    b = Box(ctx, n, L, len(pos))
    b.upload(pos, vel, mass)
    return b


def oracle_field(n, L, p: O.Particles, a, phi0=None):
    cs = O.sort(n, L, p)
    rho = O.deposit(n, L, p, cs)
    rhs, _ = O.make_rhs(n, L, rho, p.total_mass() / (L * L * L), ggrav(), a)
    phi, st, cyc, r0, r = O.mg_solve(n, L, rhs, phi0)
    return rho, phi, cyc


def compare_particles(box, p: O.Particles, L, tol=TOL):
    gpos, gvel = box.download()
    opos, ovel = p.by_id()
    d = min_image(gpos - opos, L)
    ex = np.linalg.norm(d) / np.linalg.norm(opos)
    ev = rel_l2(gvel, ovel)
    assert ex <= tol and ev <= tol, (ex, ev)
    return ex, ev


@pytest.mark.parametrize("n", [64])
def test_deposit_bitwise(ctx, n):
    ic = config1_ics(n, seed=1)
    b = make_box(ctx, n, 1.0, ic.pos, ic.vel, ic.mass)
    rho_g = b.deposit()
    p = O.Particles(ic.pos, ic.vel, ic.mass)
    rho_o = O.deposit(n, 1.0, p, O.sort(n, 1.0, p))
    assert np.array_equal(rho_g, rho_o), rel_l2(rho_g, rho_o)
    # deterministic across calls and re-sorts
    b.redistribute()
    assert np.array_equal(b.deposit(), rho_g)


def test_solve_grav_and_kicks_match_oracle(ctx):
    n, a = 64, 0.02
    ic = config1_ics(n, seed=1)
    b = make_box(ctx, n, 1.0, ic.pos, ic.vel, ic.mass)
    p = O.Particles(ic.pos, ic.vel, ic.mass)
    b.deposit(read_back=False)
    info = b.solve_phi(a, zero_guess=True)
    rho_o, phi_o, cyc = oracle_field(n, 1.0, p, a)
    phi_g = b.get_phi()
    assert info["vcycles"] == cyc
    assert rel_l2(mean_removed(phi_g), mean_removed(phi_o)) <= TOL
    g_g = b.grav_vector()
    g_o = O.grav_vector(n, 1.0, phi_o)
    assert rel_l2(g_g, g_o) <= TOL
    # kick-drift then kick with the same field
    dt, a_half, a_new = 1e-5, 0.021, 0.022
    b.kick_drift(dt, a, a_half)
    O.move(n, 1.0, p, g_o, dt, a, a_half, 1)
    compare_particles(b, p, 1.0)
    b.kick(dt, a_new, a_half)
    O.move(n, 1.0, p, g_o, dt, a_half, a_new, 0)
    compare_particles(b, p, 1.0)


def test_kicks_with_the_callers_acceleration(ctx):
    """moveKickDrift / moveKick take a caller-owned acc MultiFab
    (DarkMatterParticleContainer.cpp:76-112, 184-247): an acceleration computed
    outside the box (here the oracle's gravity vector of a displaced state, and a
    random field) is handed over from host memory and from device memory, and the
    kicks equal the oracle's update_dm_particle_single bit for bit.  The mixed form
    kicks with the same field rounded to FP32, within 1e-6."""
    import torch
    from nyx_gb300.pm import DarkMatterParticleContainer
    n, L, a = 32, 1.0, 0.03
    ic = config1_ics(n, seed=5)
    # a field that is not the box's own: the oracle's from other particles
    other = config1_ics(n, seed=6)
    _, phi_o, _ = oracle_field(n, L, O.Particles(other.pos, other.vel, other.mass), a)
    g_o = O.grav_vector(n, L, phi_o)
    g_r = np.random.default_rng(7).standard_normal(3 * n ** 3) * float(np.abs(g_o).max())
    dt, a_half, a_new = 2e-4, 0.0305, 0.031
    for g, on_device in ((g_o, False), (g_r, True)):
        b = make_box(ctx, n, L, ic.pos, ic.vel, ic.mass)
        dm = DarkMatterParticleContainer(b)
        acc = torch.from_numpy(g).cuda() if on_device else g.reshape(3, n, n, n)
        dm.moveKickDrift(acc, 0, dt, a, a_half)
        torch.cuda.synchronize()
        p = O.Particles(ic.pos, ic.vel, ic.mass)
        O.move(n, L, p, g, dt, a, a_half, 1)
        gpos, gvel = b.download()
        opos, ovel = p.by_id()
        assert np.array_equal(gpos, opos) and np.array_equal(gvel, ovel)
        dm.moveKick(None, 0, dt, a_new, a_half)   # the same field stays in place
        O.move(n, L, p, g, dt, a_half, a_new, 0)
        gpos, gvel = b.download()
        opos, ovel = p.by_id()
        assert np.array_equal(gpos, opos) and np.array_equal(gvel, ovel)
        assert np.array_equal(b.grav_vector(), g)
        # a solve replaces the caller's field by the box's own
        b.deposit(read_back=False)
        b.solve_phi(a, zero_guess=True)
        assert not np.array_equal(b.grav_vector(), g)
        b.close()
    bm = Box(ctx, n, L, len(ic.pos), precision="mixed")
    bm.upload(ic.pos, ic.vel, ic.mass)
    bm.set_grav_vector(g_o)
    bm.kick_drift(dt, a, a_half)
    p = O.Particles(ic.pos, ic.vel, ic.mass)
    O.move(n, L, p, g_o, dt, a, a_half, 1)
    gpos, gvel = bm.download()
    opos, ovel = p.by_id()
    dv = rel_l2(gvel, ovel)
    dx_cells = float(np.abs(min_image(gpos - opos, L)).max()) * n / L
    assert dv <= 1e-6 and dx_cells <= 1e-6, (dv, dx_cells)
    bm.close()


@pytest.mark.parametrize("reuse", [False, True])
def test_config1_step_by_step(ctx, reuse):
    """Plain PM 64^3, a 0.02 -> 0.05 in 10 equal-da steps; every GPU step starts
    from the oracle's state and is compared on rho, phi and particle state."""
    n, L = 64, 1.0
    ic = config1_ics(n, seed=1)
    p = O.Particles(ic.pos, ic.vel, ic.mass)
    pm = O.PMOracle(n, L, p, reuse_field=reuse)
    b = Box(ctx, n, L, p.np)
    sched = equal_da_schedule(0.02, 0.05, 10)
    gsched = ctx.step_schedule(0.02, 0.05, 10)
    assert np.array_equal(np.array(sched), np.array(gsched))
    if reuse:
        pm.init_field(0.02)
    for a0, a1, dt in sched:
        pos, vel = p.by_id()
        b.upload(pos, vel, ic.mass)
        if reuse:
            b.set_phi(pm.phi)
        info = b.step(a0, a1, dt, reuse_field=reuse)
        pm.step(a0, a1, dt)
        assert info["new_solve"]["vcycles"] == pm.cycles[1]
        if not reuse:
            assert info["old_solve"]["vcycles"] == pm.cycles[0]
        assert rel_l2(mean_removed(b.get_phi()), mean_removed(pm.phi)) <= TOL
        assert rel_l2(b.grav_vector(), pm.g) <= TOL
        compare_particles(b, p, L)


def test_config1_free_running_deterministic(ctx):
    n, L = 64, 1.0
    ic = config1_ics(n, seed=1)
    sched = ctx.step_schedule(0.02, 0.05, 10)
    outs = []
    for _ in range(2):
        b = Box(ctx, n, L, len(ic.pos))
        b.upload(ic.pos, ic.vel, ic.mass)
        for a0, a1, dt in sched:
            b.step(a0, a1, dt)
        outs.append(b.download())
        b.close()
    assert np.array_equal(outs[0][0], outs[1][0]) and np.array_equal(outs[0][1], outs[1][1])
    # free-running against the oracle: no chaos amplification yet at a = 0.05
    p = O.Particles(ic.pos, ic.vel, ic.mass)
    pm = O.PMOracle(n, L, p)
    for a0, a1, dt in sched:
        pm.step(a0, a1, dt)
    opos, ovel = p.by_id()
    assert np.linalg.norm(min_image(outs[0][0] - opos, L)) / np.linalg.norm(opos) <= 1e-11
    assert rel_l2(outs[0][1], ovel) <= 1e-11


@pytest.mark.parametrize("n", [4, 6, 12, 48])
def test_grid_sizes(ctx, n):
    ic = zeldovich_ics(n, 2.0, -2.0, n, 0.05, rms_disp_cells=0.3)
    p = O.Particles(ic.pos, ic.vel, ic.mass)
    pm = O.PMOracle(n, 2.0, p)
    b = make_box(ctx, n, 2.0, ic.pos, ic.vel, ic.mass)
    for a0, a1, dt in equal_da_schedule(0.05, 0.08, 2):
        info = b.step(a0, a1, dt)
        pm.step(a0, a1, dt)
        assert info["new_solve"]["vcycles"] == pm.cycles[1]
    assert rel_l2(mean_removed(b.get_phi()), mean_removed(pm.phi)) <= TOL
    compare_particles(b, p, 2.0)


def test_edge_positions_and_crowded_cell(ctx):
    """Particles on cell faces, at 0 and just below L, and 20000 in one deposit
    cell (exercises the long-segment sort path); per-particle masses."""
    n, L = 16, 1.0
    rng = np.random.default_rng(7)
    faces = np.array([[0.0, 0.0, 0.0], [np.nextafter(L, 0), 0.5, 0.5], [0.5, 0.5, 0.5],
                      [1 / 16, 2 / 16, 3 / 16], [0.03125, 0.96875, 0.5]])
    crowd = 0.3 + 0.01 * rng.random((20000, 3))
    rest = rng.random((3000, 3))
    pos = np.concatenate([faces, crowd, rest])
    vel = rng.standard_normal(pos.shape) * 10.0
    mass = rng.random(len(pos)) * 1e9 + 1e8
    b = make_box(ctx, n, L, pos, vel, mass)
    p = O.Particles(pos, vel, mass)
    rho_g = b.deposit()
    rho_o = O.deposit(n, L, p, O.sort(n, L, p))
    assert np.array_equal(rho_g, rho_o)
    pm = O.PMOracle(n, L, p)
    for a0, a1, dt in equal_da_schedule(0.1, 0.12, 2):
        b.step(a0, a1, dt)
        pm.step(a0, a1, dt)
    compare_particles(b, p, L)


def test_single_particle(ctx):
    pos = np.array([[0.3, 0.7, 0.1]])
    b = make_box(ctx, 8, 1.0, pos, np.array([[1.0, 2.0, 3.0]]), 5e9)
    rho = b.deposit()
    assert rho.sum() * (1.0 / 8) ** 3 == pytest.approx(5e9, rel=1e-14)
    info = b.solve_phi(0.5, zero_guess=True)
    assert info["resnorm"] <= 1e-10 * max(info["bnorm"], info["resnorm0"])


def test_invalid_arguments_are_errors(ctx):
    with pytest.raises(NyxPMError):
        Box(ctx, 9, 1.0, 10)          # 9 is not m*2^k with m <= 8
    with pytest.raises(NyxPMError):
        Box(ctx, 16, 0.0, 10)
    with pytest.raises(NyxPMError):
        Box(ctx, 16, 1.0, 0)
    b = Box(ctx, 16, 1.0, 4)
    with pytest.raises(NyxPMError):
        b.deposit()                   # nothing uploaded
    with pytest.raises(NyxPMError):
        b.upload(np.full((4, 3), np.nan), np.zeros((4, 3)), 1.0)
    with pytest.raises(NyxPMError):
        b.step(0.1, 0.2, 1e-3, reuse_field=True)


def test_zeldovich_pancake_on_gpu(ctx):
    """The reference's known answer through the GPU path."""
    d = load_zeldovich()
    pos, vel, mass, X, L, n, h = zeldovich_particles(d)
    from nyx_gb300.pm import Context
    c = Context(h=h)
    b = Box(c, n, L, len(pos))
    b.upload(pos, vel, mass)
    a = d["stops"][0]["a"]
    b.init_field(a)
    stop = d["stops"][1]
    for a0, a1, dt in zeldovich_schedule(a, stop["a"], h):
        b.step(a0, a1, dt, reuse_field=True)
        a = a1
    ps, vs = b.download()
    ex, ev = zeldovich_errors(ps, vs, stop, X, L, a)
    assert ex < 0.03 and ev < 0.05, (ex, ev)
    b.close()
    c.close()


def test_config2_full_size_properties(ctx):
    """256^3 particles on a 256^3 grid (the plain GPU config): deposit parity,
    mass and momentum conservation, solve parity, determinism."""
    n, L = 256, 1.0
    ic = zeldovich_ics(n, L, -2.0, 2, 0.02, rms_disp_cells=0.2)
    b = make_box(ctx, n, L, ic.pos, ic.vel, ic.mass)
    rho_g = b.deposit()
    p = O.Particles(ic.pos, ic.vel, ic.mass)
    rho_o = O.deposit(n, L, p, O.sort(n, L, p))
    assert np.array_equal(rho_g, rho_o)
    assert rho_g.sum() * (L / n) ** 3 == pytest.approx(ic.mass * len(ic.pos), rel=1e-12)
    info = b.solve_phi(0.02, zero_guess=True)
    rhs, _ = O.make_rhs(n, L, rho_o, p.total_mass() / (L * L * L), ggrav(), 0.02)
    phi_o, st, cyc, r0, r = O.mg_solve(n, L, rhs)
    assert info["vcycles"] == cyc
    assert rel_l2(mean_removed(b.get_phi()), mean_removed(phi_o)) <= TOL
    sched = ctx.step_schedule(0.02, 0.5, 50)
    mom0 = ic.vel.sum(axis=0) * 0.02
    for a0, a1, dt in sched[:2]:
        b.step(a0, a1, dt)
    pos, vel = b.download()
    scale = np.abs(vel).sum() * sched[1][1]
    assert np.abs(vel.sum(axis=0) * sched[1][1] - mom0).max() < 1e-9 * scale
    b2 = make_box(ctx, n, L, ic.pos, ic.vel, ic.mass)
    b2.deposit(read_back=False)
    b2.solve_phi(0.02, zero_guess=True)
    for a0, a1, dt in sched[:2]:
        b2.step(a0, a1, dt)
    pos2, vel2 = b2.download()
    assert np.array_equal(pos, pos2) and np.array_equal(vel, vel2)


@pytest.mark.parametrize("precision", ["fp64", "mixed"])
def test_vcycle_cap_reports_not_converged(precision):
    """A solve that reaches max_vcycles above the tolerance returns
    NYXPM_NOT_CONVERGED (where MLMG aborts) and leaves a usable field; the FP64
    form stops at the same V-cycle as the oracle with the same cap."""
    from nyx_gb300.pm import Context
    n = 32
    ic = config1_ics(n, seed=2)
    c2 = Context(device=0, max_vcycles=2)
    b = Box(c2, n, 1.0, len(ic.pos), precision=precision)
    b.upload(ic.pos, ic.vel, ic.mass)
    b.deposit(read_back=False)
    with pytest.raises(NyxPMError) as e:
        b.solve_phi(0.02, zero_guess=True)
    assert e.value.status == 4 and "max_vcycles" in str(e.value)
    g = b.grav_vector()
    assert np.all(np.isfinite(g)) and np.abs(g).max() > 0
    if precision == "fp64":
        p = O.Particles(ic.pos, ic.vel, ic.mass)
        rho = O.deposit(n, 1.0, p, O.sort(n, 1.0, p))
        rhs, _ = O.make_rhs(n, 1.0, rho, p.total_mass(), ggrav(), 0.02)
        phi_o, st, cyc, r0, r = O.mg_solve(n, 1.0, rhs, None, max_cycles=2)
        assert st != 0 and cyc == 2
        assert rel_l2(mean_removed(b.get_phi()), mean_removed(phi_o)) <= TOL
    b.close()
    c2.close()


@pytest.mark.parametrize("nu1,nu2", [(1, 1), (2, 0), (0, 2), (3, 1)])
def test_smoothing_counts_match_oracle(nu1, nu2):
    """Other pre/post-smoothing counts switch the exact shortcuts of the FP64
    V-cycle on and off: the red-only restriction needs nu1 > 0, the black-only
    prolongation and the red-cell norm nu2 > 0, the norm fused with the next
    opening red sweep both.  Each combination equals the oracle run with the same
    counts, bit for bit, over three steps."""
    from nyx_gb300.pm import Context
    n, L = 32, 1.0
    ic = config1_ics(n, seed=9)
    p = O.Particles(ic.pos, ic.vel, ic.mass)
    pm = O.PMOracle(n, L, p, nu1=nu1, nu2=nu2)
    c2 = Context(device=0, nu1=nu1, nu2=nu2)
    try:
        b = Box(c2, n, L, p.np)
        b.upload(ic.pos, ic.vel, ic.mass)
        for a0, a1, dt in equal_da_schedule(0.02, 0.04, 3):
            info = b.step(a0, a1, dt)
            pm.step(a0, a1, dt)
            assert info["old_solve"]["vcycles"] == pm.cycles[0]
            assert info["new_solve"]["vcycles"] == pm.cycles[1]
            assert np.array_equal(mean_removed(b.get_phi()), mean_removed(pm.phi))
        gpos, gvel = b.download()
        opos, ovel = p.by_id()
        assert np.array_equal(gpos, opos) and np.array_equal(gvel, ovel)
        b.close()
    finally:
        c2.close()
