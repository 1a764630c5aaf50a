"""The multilevel (AMR) step on the GPU (nyxpm_amr_*) against the multilevel
oracle, on the reference's own AMR test grids (Exec/ParticleOnlyTest:
fixed_grids.mass, particle_file.mass) and on Zel'dovich particles.

Tolerances: particle levels and boxes exactly; the deposit to 1e-13 (the GPU
adds corner masses with atomics, in another order); phi and g to 1e-9 relative
and equal V-cycle counts (the solve stops at rel_tol 1e-10); positions to 1e-12
and the velocity change of a step to 1e-8.
"""
from __future__ import annotations

import os

import numpy as np
import pytest

from nyx_gb300.amr import AmrHierarchy, regrid_file_boxes
from nyx_gb300.ics import zeldovich_ics
from nyx_gb300.pm import Box, Context, NyxPMError
from oracle import oracle as O
from tests.conftest import gpu_available

pytestmark = [pytest.mark.gpu, pytest.mark.skipif(not gpu_available(), reason="no GPU")]

GOLDEN = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden")


def _rel(a, b):
    return float(np.linalg.norm(a - b) / max(np.linalg.norm(b), 1e-300))


def reference_boxes():
    with open(os.path.join(GOLDEN, "particle_only_fixed_grids.mass")) as f:
        return regrid_file_boxes(f)


@pytest.fixture(scope="module")
def ctx():
    c = Context(device=0)
    yield c


def _cfl_step(ctx, vel, h, a0=0.05, frac=0.4):
    dt = frac * h * a0 / float(np.abs(vel).max())
    return a0, ctx.integrate_comoving_a(a0, dt), dt


def _nboxes(boxes):
    return sum(len(lv) for lv in boxes)


def test_parts_of_the_step_match_the_oracle(ctx):
    n0, L = 16, 1.0
    boxes = reference_boxes()
    ic = zeldovich_ics(n0, L, -2.0, 31, 0.05, rms_disp_cells=0.6)
    rng = np.random.default_rng(5)
    pos = np.concatenate([ic.pos, (np.array([28.0, 20.0, 28.0]) / 64 + rng.normal(0, 0.03, (1500, 3))) % 1.0])
    vel = np.concatenate([ic.vel, rng.normal(0, np.abs(ic.vel).std(), (1500, 3))])
    mass = rng.random(len(pos)) + 0.5
    H = AmrHierarchy(ctx, n0, L, boxes, len(pos))
    H.upload(pos, vel, mass)
    p = O.Particles(pos, vel, mass)
    A = O.AmrOracle(n0, L, boxes, p)
    lev, box = H.assign()
    olev, obox = A.assign()
    np.testing.assert_array_equal(lev, olev)
    np.testing.assert_array_equal(box, obox)
    assert set(np.unique(lev)) == {0, 1, 2}
    H.deposit()
    A.deposit()
    for b in range(-1, _nboxes(boxes)):
        assert _rel(H.field("rho", b), A.field("rho", b)) <= 1e-13, b
    h0 = L / n0
    assert abs(H.field("rho").sum() * h0 ** 3 - mass.sum()) <= 1e-12 * mass.sum()
    a = 0.05
    info = H.solve(a)
    st, cycles, _, _ = A.solve(a)
    assert st == 0 and info["vcycles"] == cycles
    for b in range(-1, _nboxes(boxes)):
        ph, po = H.field("phi", b), A.field("phi", b)
        assert _rel(ph, po) <= 1e-9, b
    H.grav_vector()
    A.grav()
    for b in range(-1, _nboxes(boxes)):
        for c in ("gx", "gy", "gz"):
            assert _rel(H.field(c, b), A.field(c, b)) <= 1e-9, (b, c)
    a0, a1, dt = _cfl_step(ctx, vel, L / (4 * n0))
    H.kick(dt, a0, 0.5 * (a0 + a1), True)
    assert A.move(dt, a0, 0.5 * (a0 + a1), 1) == 0
    xg, vg = H.download()
    assert _rel(xg, p.pos()) <= 1e-12
    assert _rel(vg - vel, p.vel() - vel) <= 1e-8


# two level-1 boxes sharing a face (their ghosts copy each other's cells) and a
# level-2 box whose parents lie in both (the prolongation's general path)
TOUCHING = [[((8, 8, 8), (15, 23, 23)), ((16, 8, 8), (23, 23, 23))], [((28, 20, 20), (35, 27, 27))]]


# three refined levels (the most the library takes), nested about the centre
THREE = [[((8, 8, 8), (23, 23, 23))], [((20, 20, 20), (43, 43, 43))], [((44, 44, 44), (83, 83, 83))]]


@pytest.mark.parametrize("seed, layout", [(41, "reference"), (42, "reference"), (43, "touching"),
                                          (44, "three")])
def test_steps_match_the_oracle(ctx, seed, layout):
    n0, L = 16, 1.0
    boxes = {"reference": reference_boxes(), "touching": TOUCHING, "three": THREE}[layout]
    ic = zeldovich_ics(n0, L, -2.0, seed, 0.05, rms_disp_cells=0.5)
    pos, vel = ic.pos, ic.vel
    if layout == "three":
        rng = np.random.default_rng(3)
        pos = np.concatenate([pos, (0.5 + rng.normal(0, 0.05, (3000, 3))) % 1.0])
        vel = np.concatenate([vel, np.zeros((3000, 3))])
    H = AmrHierarchy(ctx, n0, L, boxes, len(pos))
    H.upload(pos, vel, ic.mass)
    p = O.Particles(pos, vel, ic.mass)
    A = O.AmrOracle(n0, L, boxes, p)
    a0, a1, dt = _cfl_step(ctx, vel, L / (2 ** len(boxes) * n0))
    for _ in range(3):
        v_before = p.vel().copy()
        info = H.step(a0, a1, dt)
        assert A.step(a0, a1, dt) == 0
        assert info["old_solve"]["vcycles"] == A.cycles[0]
        assert info["new_solve"]["vcycles"] == A.cycles[1]
        xg, vg = H.download()
        assert _rel(xg, p.pos()) <= 1e-12
        assert _rel(vg - v_before, p.vel() - v_before) <= 1e-8
        a0, a1 = a1, ctx.integrate_comoving_a(a1, dt)


def test_reference_particle_test(ctx):
    """inputs.mass.nosub's eight massive particles on its fixed grids, a = 1."""
    data = np.loadtxt(os.path.join(GOLDEN, "particle_only_particle_file.mass"), skiprows=1)
    pos, mass, vel = data[:, 0:3], data[:, 3], data[:, 4:7]
    boxes = reference_boxes()
    H = AmrHierarchy(ctx, 16, 32.0, boxes, len(pos))
    H.upload(pos, vel, mass)
    p = O.Particles(pos, vel, mass)
    A = O.AmrOracle(16, 32.0, boxes, p)
    for _ in range(3):
        H.step(1.0, 1.0, 0.05)
        assert A.step(1.0, 1.0, 0.05) == 0
    xg, vg = H.download()
    assert _rel(xg, p.pos()) <= 1e-13
    assert _rel(vg - vel, p.vel() - vel) <= 1e-8


def test_two_full_domain_levels_equal_single_level_box(ctx):
    n0, L = 8, 1.0
    ic = zeldovich_ics(4 * n0, L, -2.0, 17, 0.05, rms_disp_cells=0.3)
    H = AmrHierarchy(ctx, n0, L, [[((0, 0, 0), (2 * n0 - 1,) * 3)], [((0, 0, 0), (4 * n0 - 1,) * 3)]],
                     len(ic.pos))
    H.upload(ic.pos, ic.vel, ic.mass)
    B = Box(ctx, 4 * n0, L, len(ic.pos))
    B.upload(ic.pos, ic.vel, ic.mass)
    a0, a1, dt = _cfl_step(ctx, ic.vel, L / (4 * n0))
    H.step(a0, a1, dt)
    B.step(a0, a1, dt)
    xa, va = H.download()
    xb, vb = B.download()
    assert _rel(xa, xb) <= 1e-14
    assert _rel(va - ic.vel, vb - ic.vel) <= 1e-8
    B.close()


def test_full_domain_level_equals_single_level_box(ctx):
    n0, L = 16, 1.0
    ic = zeldovich_ics(2 * n0, L, -2.0, 11, 0.05, rms_disp_cells=0.3)
    H = AmrHierarchy(ctx, n0, L, [[((0, 0, 0), (2 * n0 - 1,) * 3)]], len(ic.pos))
    H.upload(ic.pos, ic.vel, ic.mass)
    B = Box(ctx, 2 * n0, L, len(ic.pos))
    B.upload(ic.pos, ic.vel, ic.mass)
    a0, a1, dt = _cfl_step(ctx, ic.vel, L / (2 * n0))
    H.step(a0, a1, dt)
    B.step(a0, a1, dt)
    xa, va = H.download()
    xb, vb = B.download()
    assert _rel(xa, xb) <= 1e-14
    assert _rel(va - ic.vel, vb - ic.vel) <= 1e-8
    B.close()


def test_one_level_equals_single_level_box(ctx):
    n0, L = 16, 1.0
    ic = zeldovich_ics(n0, L, -2.0, 12, 0.05, rms_disp_cells=0.3)
    H = AmrHierarchy(ctx, n0, L, [], len(ic.pos))
    H.upload(ic.pos, ic.vel, ic.mass)
    B = Box(ctx, n0, L, len(ic.pos))
    B.upload(ic.pos, ic.vel, ic.mass)
    a0, a1, dt = _cfl_step(ctx, ic.vel, L / n0)
    H.step(a0, a1, dt)
    B.step(a0, a1, dt)
    xa, va = H.download()
    xb, vb = B.download()
    assert _rel(xa, xb) <= 1e-14
    assert _rel(va - ic.vel, vb - ic.vel) <= 1e-8
    B.close()


@pytest.mark.parametrize("boxes", [
    [[((1, 0, 0), (8, 7, 7))]],
    [[((0, 0, 0), (7, 7, 7)), ((6, 6, 6), (9, 9, 9))]],
    [[((0, 0, 0), (7, 7, 7))], [((0, 0, 0), (7, 7, 7))]],
    [[((0, 0, 0), (33, 7, 7))]],
])
def test_bad_grids_are_refused(ctx, boxes):
    with pytest.raises(NyxPMError):
        AmrHierarchy(ctx, 16, 1.0, boxes, 10)


def test_a_particle_outrunning_its_ghost_cells_is_reported(ctx):
    # one particle at the centre of the refined box, moving 12 of its cells in one
    # step: its closing kick would read 3 cells beyond the box
    H = AmrHierarchy(ctx, 16, 1.0, [[((8, 8, 8), (23, 23, 23))]], 1)
    pos = np.array([[0.5, 0.5, 0.5]])
    vel = np.array([[12.0 / 32 / 0.1, 0.0, 0.0]])
    H.upload(pos, vel, 1.0)
    with pytest.raises(NyxPMError, match="ghost"):
        H.step(1.0, 1.0, 0.1)
