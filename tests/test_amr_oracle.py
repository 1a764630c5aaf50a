"""The multilevel (AMR) oracle (oracle/pm_amr_oracle.cpp) on the CPU.

The reference's multilevel deposit and composite solve are AMReX's and absent
from its tree, so the oracle is pinned by properties that hold for any correct
composite PM step rather than by golden vectors:
* a level-1 box covering the whole domain gives the single-level step at twice
  the resolution (the composite V-cycle is then a V-cycle of the finer grid);
* one level gives the single-level step;
* the multilevel deposit conserves mass exactly, wherever the particles sit;
* refinement moves the forces inside a refined box toward a uniformly fine solve;
* grids that break the rules (alignment, overlap, nesting) are refused.

Fixtures: tests/golden/particle_only_fixed_grids.mass and
particle_only_particle_file.mass are the reference's own AMR particle test
inputs (Exec/ParticleOnlyTest/fixed_grids.mass and particle_file.mass, used by
inputs.mass.nosub: 16^3 base cells on a 32-unit box, 2 refined levels).
"""
from __future__ import annotations

import os

import numpy as np
import pytest

from nyx_gb300.amr import regrid_file_boxes
from nyx_gb300.ics import zeldovich_ics
from oracle import oracle as O

GOLDEN = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden")


def _rel(a, b):
    return float(np.linalg.norm(a - b) / max(np.linalg.norm(b), 1e-300))


def _cfl_step(vel, h, a0=0.05, frac=0.4):
    """(a0, a1, dt) moving the fastest particle frac of a cell of size h."""
    dt = frac * h * a0 / float(np.abs(vel).max())
    return a0, O.lib().orc_integrate_a(1.0, 0.0, 0.675, a0, dt), dt


def reference_boxes():
    with open(os.path.join(GOLDEN, "particle_only_fixed_grids.mass")) as f:
        return regrid_file_boxes(f)


def test_regrid_file_boxes_are_refined_and_nested():
    boxes = reference_boxes()
    assert boxes == [[((12, 6, 12), (25, 19, 27)), ((0, 0, 12), (7, 7, 19)), ((26, 26, 12), (31, 31, 19))],
                     [((28, 20, 28), (41, 33, 37))]]
    p = O.Particles(np.full((1, 3), 1.0), np.zeros((1, 3)), 1.0)
    O.AmrOracle(16, 32.0, boxes, p)   # accepted: aligned, disjoint, nested


def test_regrid_file_forms():
    """Regrid files as AMReX writes and reads them: the level count, then per level
    the box count and the boxes ((lo) (hi) (type)), spaces anywhere, each box in the
    index space of the level below; a box of coarse cells lo..hi becomes the fine
    cells 2 lo .. 2 hi + 1."""
    text = ["1", "2", "((0,0,0) (3,3,3) (0,0,0))", "(( 4 , 6 , 8 )   ( 5,7,9 ) ( 0, 0, 0 ))"]
    assert regrid_file_boxes(text) == [[((0, 0, 0), (7, 7, 7)), ((8, 12, 16), (11, 15, 19))]]
    text = ["3", "1", "((2,2,2) (5,5,5) (0,0,0))", "1", "((6,6,6) (9,9,9) (0,0,0))", "1",
            "((14,14,14) (17,17,17) (0,0,0))"]
    boxes = regrid_file_boxes(text)
    assert boxes == [[((4, 4, 4), (11, 11, 11))], [((12, 12, 12), (19, 19, 19))],
                     [((28, 28, 28), (35, 35, 35))]]
    p = O.Particles(np.full((1, 3), 0.5), np.zeros((1, 3)), 1.0)
    O.AmrOracle(8, 1.0, boxes, p)   # three refined levels, nested


def test_full_domain_level_equals_single_level_at_twice_the_resolution():
    n0, L = 16, 1.0
    ic = zeldovich_ics(2 * n0, L, -2.0, 11, 0.05, rms_disp_cells=0.3)
    a0, a1, dt = _cfl_step(ic.vel, L / (2 * n0))
    pa = O.Particles(ic.pos, ic.vel, ic.mass)
    ps = O.Particles(ic.pos, ic.vel, ic.mass)
    A = O.AmrOracle(n0, L, [[((0, 0, 0), (2 * n0 - 1,) * 3)]], pa)
    assert A.step(a0, a1, dt) == 0
    assert np.all(A.lev == 1)
    S = O.PMOracle(2 * n0, L, ps)
    S.step(a0, a1, dt)
    xa, va = pa.by_id()
    xs, vs = ps.by_id()
    # the solves stop at 1e-10 from different guesses (the multilevel new-time
    # solve starts from zero): the velocity change agrees to that tolerance
    assert _rel(xa, xs) < 1e-14
    assert _rel(va - ic.vel, vs - ic.vel) < 1e-8
    assert A.cycles[0] == S.cycles[0]


def test_two_full_domain_levels_equal_single_level_at_four_times_the_resolution():
    n0, L = 8, 1.0
    ic = zeldovich_ics(4 * n0, L, -2.0, 17, 0.05, rms_disp_cells=0.3)
    a0, a1, dt = _cfl_step(ic.vel, L / (4 * n0))
    pa = O.Particles(ic.pos, ic.vel, ic.mass)
    ps = O.Particles(ic.pos, ic.vel, ic.mass)
    A = O.AmrOracle(n0, L, [[((0, 0, 0), (2 * n0 - 1,) * 3)], [((0, 0, 0), (4 * n0 - 1,) * 3)]], pa)
    assert A.step(a0, a1, dt) == 0
    assert np.all(A.lev == 2)
    S = O.PMOracle(4 * n0, L, ps)
    S.step(a0, a1, dt)
    xa, va = pa.by_id()
    xs, vs = ps.by_id()
    assert _rel(xa, xs) < 1e-14
    assert _rel(va - ic.vel, vs - ic.vel) < 1e-8


THREE = [[((8, 8, 8), (23, 23, 23))], [((20, 20, 20), (43, 43, 43))], [((44, 44, 44), (83, 83, 83))]]


def test_three_refined_levels_conserve_mass_and_step():
    n0, L = 16, 1.0
    rng = np.random.default_rng(3)
    ic = zeldovich_ics(n0, L, -2.0, 44, 0.05, rms_disp_cells=0.5)
    pos = np.concatenate([ic.pos, (0.5 + rng.normal(0, 0.05, (3000, 3))) % 1.0])
    vel = np.concatenate([ic.vel, np.zeros((3000, 3))])
    p = O.Particles(pos, vel, float(ic.mass))
    A = O.AmrOracle(n0, L, THREE, p)
    lev, _ = A.assign()
    assert set(np.unique(lev)) == {0, 1, 2, 3}
    A.deposit()
    assert abs(A.total_mass() - float(ic.mass) * len(pos)) <= 1e-13 * float(ic.mass) * len(pos)
    a0, a1, dt = _cfl_step(vel, L / (8 * n0))
    assert A.step(a0, a1, dt) == 0
    assert A.cycles[0] < 20 and A.cycles[1] < 20


def test_one_level_equals_single_level():
    n0, L = 16, 1.0
    ic = zeldovich_ics(n0, L, -2.0, 12, 0.05, rms_disp_cells=0.3)
    a0, a1, dt = _cfl_step(ic.vel, L / n0)
    pa = O.Particles(ic.pos, ic.vel, ic.mass)
    ps = O.Particles(ic.pos, ic.vel, ic.mass)
    A = O.AmrOracle(n0, L, [], pa)
    assert A.step(a0, a1, dt) == 0
    S = O.PMOracle(n0, L, ps)
    S.step(a0, a1, dt)
    xa, va = pa.by_id()
    xs, vs = ps.by_id()
    assert _rel(xa, xs) < 1e-14
    assert _rel(va - ic.vel, vs - ic.vel) < 1e-8


@pytest.mark.parametrize("seed", [13, 14])
def test_deposit_conserves_mass_on_the_reference_grids(seed):
    n0, L = 16, 1.0
    rng = np.random.default_rng(seed)
    # particles everywhere, with a cluster straddling the level-2 box's faces
    pos = np.concatenate([rng.random((3000, 3)) * L,
                          np.array([28.0, 20.0, 28.0]) / 64 * L + rng.normal(0, 0.02, (2000, 3))]) % L
    mass = rng.random(len(pos)) + 0.5
    p = O.Particles(pos, np.zeros_like(pos), mass)
    A = O.AmrOracle(n0, L, reference_boxes(), p)
    lev, _ = A.assign()
    assert set(np.unique(lev)) == {0, 1, 2}
    A.deposit()
    assert abs(A.total_mass() - mass.sum()) <= 1e-13 * mass.sum()
    # the covered coarse cells hold the average of their children
    rho0 = A.field("rho")
    rho1 = A.field("rho", 0)      # level-1 box (12,6,12)-(25,19,27)
    sub = rho1.reshape(8, 2, 7, 2, 7, 2).mean(axis=(1, 3, 5))
    np.testing.assert_allclose(rho0[6:14, 3:10, 6:13], sub, rtol=1e-14, atol=0)


def test_refinement_moves_forces_toward_the_fine_solution():
    n0, L = 16, 1.0
    ic = zeldovich_ics(2 * n0, L, -2.0, 21, 0.05, rms_disp_cells=0.6)

    def accel_single(n):
        p = O.Particles(ic.pos, ic.vel * 0, ic.mass)
        S = O.PMOracle(n, L, p)
        S.init_field(1.0)
        O.lib().orc_move(n, L, p.np, p.x, p.y, p.z, p.vx, p.vy, p.vz, S.g, 2.0, 1.0, 1.0, 0)
        return p.by_id()[1]

    p = O.Particles(ic.pos, ic.vel * 0, ic.mass)
    A = O.AmrOracle(n0, L, [[((8, 8, 8), (23, 23, 23))], [((20, 20, 20), (43, 43, 43))]], p, rel_tol=1e-12)
    lev, _ = A.assign()
    A.deposit()
    st, cycles, _, _ = A.solve(1.0)
    assert st == 0 and cycles < 20
    A.grav()
    assert A.move(2.0, 1.0, 1.0, 0) == 0
    amr = p.by_id()[1]
    fine, coarse = accel_single(4 * n0), accel_single(n0)
    s = lev == 2
    err_amr = np.linalg.norm(amr[s] - fine[s]) / np.linalg.norm(fine[s])
    err_coarse = np.linalg.norm(coarse[s] - fine[s]) / np.linalg.norm(fine[s])
    assert err_amr < 0.35 * err_coarse, (err_amr, err_coarse)
    s0 = lev == 0
    np.testing.assert_allclose(np.linalg.norm(amr[s0] - coarse[s0]) / np.linalg.norm(coarse[s0]), 0, atol=0.05)


def test_reference_particle_test_runs_on_its_grids():
    """inputs.mass.nosub's eight massive particles on its fixed grids (a = 1)."""
    data = np.loadtxt(os.path.join(GOLDEN, "particle_only_particle_file.mass"), skiprows=1)
    pos, mass, vel = data[:, 0:3], data[:, 3], data[:, 4:7]
    p = O.Particles(pos, vel, mass)
    A = O.AmrOracle(16, 32.0, reference_boxes(), p, rel_tol=1e-10)
    lev, _ = A.assign()
    assert list(lev) == [1, 0, 0, 0, 0, 0, 1, 1]
    v0 = p.vel().copy()
    for _ in range(3):
        assert A.step(1.0, 1.0, 0.05) == 0
    m = mass[:, None]
    # a composite PM step does not conserve momentum exactly (a particle whose
    # cloud straddles a coarse/fine face feels a self-force of a few percent of
    # G m / h^2); the net change stays small against the sum of |m dv|
    dmv = m * (p.vel() - v0)
    assert np.abs(dmv.sum(axis=0)).max() < 0.1 * np.abs(dmv).sum()


@pytest.mark.parametrize("pair", [(0.4, 0.6), (0.24, 0.76), (0.26, 0.74), (0.1, 0.9)])
def test_mirror_pairs_feel_opposite_forces(pair):
    """Two equal masses placed mirror-symmetrically about the centre of a centred
    refined box: the deposit, the composite solve and the interpolation keep the
    symmetry, so the forces are opposite to round-off (inside, outside and across
    the coarse/fine faces at 0.25 and 0.75)."""
    pos = np.array([[pair[0], 0.5, 0.5], [pair[1], 0.5, 0.5]])
    p = O.Particles(pos, np.zeros_like(pos), 1.0)
    A = O.AmrOracle(16, 1.0, [[((8, 8, 8), (23, 23, 23))]], p, rel_tol=1e-13)
    A.assign()
    A.deposit()
    A.solve(1.0)
    A.grav()
    A.move(2.0, 1.0, 1.0, 0)
    f = p.vel()
    assert abs(f[0, 0]) > 0
    assert abs(f[0, 0] + f[1, 0]) <= 1e-9 * abs(f[0, 0])
    assert np.abs(f[:, 1:]).max() <= 1e-12 * abs(f[0, 0])


@pytest.mark.parametrize("boxes, why", [
    ([[((1, 0, 0), (8, 7, 7))]], "aligned"),
    ([[((0, 0, 0), (7, 7, 7)), ((6, 6, 6), (9, 9, 9))]], "overlap"),
    ([[((0, 0, 0), (7, 7, 7))], [((0, 0, 0), (7, 7, 7))]], "nested"),
    ([[((0, 0, 0), (33, 7, 7))]], "outside"),
])
def test_bad_grids_are_refused(boxes, why):
    p = O.Particles(np.full((1, 3), 0.5), np.zeros((1, 3)), 1.0)
    with pytest.raises(ValueError, match=why):
        O.AmrOracle(16, 1.0, boxes, p)
