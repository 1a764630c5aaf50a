"""CPU tests of the FP64 oracle: pinned against the reference's own
Zel'dovich pancake (analytic solution from zeldovich.py, ICs from the
reference generator) and against the physics known answers the PM path must
satisfy.  No GPU needed."""
from __future__ import annotations

import math

import numpy as np
import pytest

from oracle import oracle as O
from nyx_gb300.ics import Cosmology, GCONST, zeldovich_ics
from tests.pm_cases import (config1_ics, equal_da_schedule, load_zeldovich, mean_removed, rel_l2,
                            zeldovich_errors, zeldovich_particles, zeldovich_schedule)


def test_gconst_matches_constants_cosmo():
    # Source/Driver/constants_cosmo.H:15-16 -> about 4.3e-9 (km/s)^2 Mpc / M_sun
    assert O.gconst() == pytest.approx(GCONST, rel=0, abs=0)
    assert 4.2e-9 < O.gconst() < 4.4e-9


def test_zeldovich_generator_convention():
    """Our pancake construction reproduces the reference generator's particles."""
    d = load_zeldovich()
    P = d["params"]
    import importlib.util
    L, k, offset, H0 = P["box_length"], P["k"], P["offset"], P["H_0"]
    zi, zc = P["initial_z"], P["caustic_z"]
    a_i = 1.0 / (1.0 + zi)
    # the generator's lattice: -L/10 + i*spacing + half_cell, filtered to the box
    n1 = 128
    spacing = np.float32(L) / n1  # (float) box_length / num_particles_1d
    spacing = float(spacing)
    half = (L / n1) / 2.0
    for row in d["generator_sample"][:64]:
        x, y, z, m, vx, vy, vz = row
        # recover the lattice coordinate of x: q_lat = x - perturbation(q)
        # Newton on q: x = q - D sin(k(q+offset))/k
        D = (1.0 + zc) / (1.0 + zi)
        q = x
        for _ in range(50):
            f = q - D * math.sin(k * (q + offset)) / k - x
            fp = 1.0 - D * math.cos(k * (q + offset))
            q -= f / fp
        v_expect = -H0 * (1.0 + zc) * math.sqrt(1.0 + zi) * math.sin(k * (q + offset)) / k * a_i
        assert vx == pytest.approx(v_expect, rel=1e-9, abs=1e-9)
        assert vy == 0.0 and vz == 0.0
        # y, z sit on the lattice
        iy = (y + L / 10.0 - half) / spacing
        assert abs(iy - round(iy)) < 1e-6
    assert d["generator_particle_count"] == 2097152


def test_deposit_conserves_mass_and_uniform_lattice():
    ic = zeldovich_ics(16, 1.0, -2.0, 3, 0.02, rms_disp_cells=0.0)
    p = O.Particles(ic.pos, ic.vel, ic.mass)
    cs = O.sort(16, 1.0, p)
    rho = O.deposit(16, 1.0, p, cs)
    rho_bar = ic.mass * 16 ** 3 / 1.0
    assert np.allclose(rho, rho_bar, rtol=1e-14, atol=0)
    rhs, mean = O.make_rhs(16, 1.0, rho, p.total_mass(), -4 * math.pi * O.gconst(), 0.02)
    assert np.abs(rhs).max() == 0.0
    ic = config1_ics(32, seed=5)
    p = O.Particles(ic.pos, ic.vel, ic.mass)
    cs = O.sort(32, 1.0, p)
    rho = O.deposit(32, 1.0, p, cs)
    assert rho.sum() * (1.0 / 32) ** 3 == pytest.approx(p.total_mass(), rel=1e-13)


def test_sort_is_stable_and_segments_match_keys():
    rng = np.random.default_rng(0)
    n = 8
    pos = rng.random((500, 3))
    pos[:50] = pos[0]  # a crowded key
    p = O.Particles(pos, np.zeros_like(pos), 1.0)
    cs = O.sort(n, 1.0, p)
    keys = (np.floor(p.x * n + 0.5).astype(int) % n) + n * ((np.floor(p.y * n + 0.5).astype(int) % n)
                                                           + n * (np.floor(p.z * n + 0.5).astype(int) % n))
    assert np.all(np.diff(keys) >= 0)
    for K in range(n ** 3):
        seg = p.id[cs[K]:cs[K + 1]]
        assert np.all(np.diff(seg) > 0)  # stable: ids (initial order) increasing
        assert np.all(keys[cs[K]:cs[K + 1]] == K)


def test_multigrid_converges_and_matches_spectral_solution():
    n, L = 32, 1.0
    rng = np.random.default_rng(1)
    rhs = rng.standard_normal(n ** 3)
    rhs -= rhs.mean()
    phi, st, cyc, r0, r = O.mg_solve(n, L, rhs, rel_tol=1e-12)
    assert st == 0 and r <= 1e-12 * max(np.abs(rhs).max(), r0)
    assert 3 <= cyc <= 20
    # exact discrete solution by FFT of the 7-point periodic Laplacian
    h = L / n
    k = np.fft.fftfreq(n) * 2 * np.pi
    lam = (2 * np.cos(k)[:, None, None] - 2 + 2 * np.cos(k)[None, :, None] - 2
           + 2 * np.cos(k)[None, None, :] - 2) / h ** 2
    lam[0, 0, 0] = 1.0
    R = np.fft.fftn(rhs.reshape(n, n, n))
    Phi = R / lam
    Phi[0, 0, 0] = 0
    exact = np.real(np.fft.ifftn(Phi)).ravel()
    assert rel_l2(mean_removed(phi), mean_removed(exact)) < 1e-10


def test_multigrid_odd_bottom_and_small_grids():
    for n in (2, 3, 4, 6, 12, 24, 48):
        rng = np.random.default_rng(n)
        rhs = rng.standard_normal(n ** 3)
        rhs -= rhs.mean()
        phi, st, cyc, r0, r = O.mg_solve(n, 1.0, rhs, rel_tol=1e-11)
        assert st == 0, n
        assert r <= 1e-11 * max(np.abs(rhs).max(), r0) * (1 + 1e-12), n
    assert O.mg_levels(9) == 0 and O.mg_levels(18) == 0 and O.mg_levels(20) == 3
    assert O.mg_levels(256) == 7 and O.mg_levels(48) == 5


def test_two_particle_attraction_sign():
    """g = +grad(phi_N) points toward the mass (rhs = -4 pi G (rho - rho_bar) / a)."""
    n, L = 16, 1.0
    pos = np.array([[0.40, 0.5, 0.5], [0.60, 0.5, 0.5]])
    p = O.Particles(pos, np.zeros_like(pos), 1e10)
    pm = O.PMOracle(n, L, p)
    pm.init_field(1.0)
    g = pm.g.reshape(3, n, n, n)
    # interpolate at each particle via a zero-length kick: v gains dt/2 * g
    O.move(n, L, p, pm.g, 1.0, 1.0, 1.0, 0)
    (x0, x1), (v0, v1) = p.by_id()[0][:, 0], p.by_id()[1][:, 0]
    assert v0 > 0 and v1 < 0           # each moves toward the other
    assert v0 == pytest.approx(-v1, rel=1e-10)
    assert np.abs(g).max() > 0


def test_momentum_conservation_and_schedule():
    ic = config1_ics(32, seed=2)
    p = O.Particles(ic.pos, ic.vel, ic.mass)
    pm = O.PMOracle(32, 1.0, p)
    mom0 = p.vel().sum(axis=0)
    sched = equal_da_schedule(0.02, 0.05, 4)
    for a0, a1, dt in sched:
        st = pm.step(a0, a1, dt)
        assert st == 0
    # total momentum (a*v summed) drifts only by force asymmetry of CIC+central differences
    mom = p.vel().sum(axis=0) * sched[-1][1]
    scale = np.abs(p.vel()).sum() * sched[-1][1]
    assert np.abs(mom - mom0 * 0.02).max() < 1e-10 * scale
    assert sched[-1][1] == pytest.approx(0.05, rel=2e-3)


def test_a_of_t_matches_eds_analytic():
    h = 0.675
    H0 = 100 * h
    a0 = 0.02
    # EdS: a(t) = (a0^{3/2} + 3/2 H0 dt)^{2/3}
    for dt in (1e-6, 1e-5, 1e-4):
        an = O.integrate_a(1.0, 0.0, h, a0, dt)
        exact = (a0 ** 1.5 + 1.5 * H0 * dt) ** (2.0 / 3.0)
        assert an == pytest.approx(exact, rel=1e-7)
    dt = O.dt_for_da(1.0, 0.0, h, 0.02, 0.023, 2e-5)
    exact = (0.023 ** 1.5 - 0.02 ** 1.5) / (1.5 * H0)
    assert dt == pytest.approx(exact, rel=2e-3)


def test_zeldovich_pancake_known_answer():
    """Pin of the oracle: the PM step reproduces the reference's analytic pancake
    (Exec/GravityTests/zeldovich_dm/analysis/zeldovich.py) before shell crossing."""
    d = load_zeldovich()
    pos, vel, mass, X, L, n, h = zeldovich_particles(d)
    p = O.Particles(pos, vel, mass)
    pm = O.PMOracle(n, L, p, h=h)
    a = d["stops"][0]["a"]
    pm.init_field(a)
    for stop in d["stops"][1:2]:
        for a0, a1, dt in zeldovich_schedule(a, stop["a"], h):
            assert pm.step(a0, a1, dt) == 0
            a = a1
        ps, vs = p.by_id()
        ex, ev = zeldovich_errors(ps, vs, stop, X, L, a)
        # PM resolution of a 32-cell wavelength: ~1-4% (a 10% change of G gives ~10%)
        assert ex < 0.03, ex
        assert ev < 0.05, ev
        assert np.abs(ps[:, 1] - pos[:, 1]).max() < 1e-12


def test_particle_time_step_limit():
    """estTimestep (NyxParticleContainer.H:329-465): velocity CFL, the acceleration
    limit and the no-particle / no-limit sentinels."""
    n, L, a, cfl = 16, 1.0, 0.1, 0.5
    dx = L / n
    g = np.zeros(3 * n ** 3)
    pos = np.array([[0.30, 0.41, 0.77], [0.9, 0.1, 0.5]])
    vel = np.array([[2.0, -3.0, 1.0], [0.0, 0.0, 0.0]])
    p = O.Particles(pos, vel, 1.0)
    assert O.est_time_step(n, L, p, g, cfl, a) == cfl / (3.0 * (n / L / a))
    p0 = O.Particles(pos, np.zeros_like(vel), 1.0)
    assert O.est_time_step(n, L, p0, g, cfl, a) == 1e50
    # acceleration at the particle's cell floor(x / dx) limits dt to 1/sqrt(|g|/dx)
    c = 4 + n * (6 + n * 12)      # cell of particle 0: (0.30, 0.41, 0.77) * 16
    g[c], g[n ** 3 + c], g[2 * n ** 3 + c] = 3.0, 4.0, 0.0
    assert O.est_time_step(n, L, p0, g, cfl, a) == 1.0 / math.sqrt(5.0 / dx)
    empty = O.Particles(np.zeros((0, 3)), np.zeros((0, 3)), 1.0)
    assert O.est_time_step(n, L, empty, g, cfl, a) == -1e50
