"""Shared inputs for the parity tests: seeded initial conditions, the
Zel'dovich pancake of the reference test, and comparison helpers."""
from __future__ import annotations

import json
import math
import os

import numpy as np

from nyx_gb300.ics import Cosmology, zeldovich_ics

HERE = os.path.dirname(os.path.abspath(__file__))
GOLDEN = os.path.join(HERE, "golden")


def rel_l2(a, b) -> float:
    a = np.asarray(a, dtype=np.float64).ravel()
    b = np.asarray(b, dtype=np.float64).ravel()
    den = np.linalg.norm(b)
    num = np.linalg.norm(a - b)
    return float(num / den) if den > 0 else float(num)


def mean_removed(f):
    f = np.asarray(f, dtype=np.float64)
    return f - f.mean()


def min_image(d, L):
    return (d + 0.5 * L) % L - 0.5 * L


def true_resnorm(box, n, L, a):
    """||rhs - L phi||_inf of the box's phi under the oracle's FP64 operator, with
    the rhs built by the oracle from the box's own density and mass offset (the
    check of a solve's residual independent of the norm the solver tracked);
    returns (resnorm, ||rhs||_inf)."""
    from oracle import oracle as O
    rhs, _ = O.make_rhs(n, L, box.deposit(), box.mass_offset(), -4.0 * math.pi * O.gconst(), a)
    _, _, _, r0, _ = O.mg_solve(n, L, rhs, box.get_phi(), max_cycles=0)
    return r0, float(np.abs(rhs).max())


def config1_ics(n=64, seed=1, slope=-2.0, a_init=0.02, fraction=1.0):
    """Plain PM, CPU-runnable config: unit box, EdS, rms displacement 0.2 cell at a=0.02."""
    return zeldovich_ics(n, 1.0, slope, seed, a_init, rms_disp_cells=0.2, fraction=fraction)


def equal_da_schedule(a0, a1, nsteps, OmM=1.0, OmR=0.0, h=0.675):
    """Oracle copy of the host schedule: equal delta-a, dt from integrate_comoving_a_to_a,
    a_new re-integrated from dt."""
    from oracle import oracle as O
    cos = Cosmology(OmM, OmR, h)
    out = []
    a = a0
    da = (a1 - a0) / nsteps
    for _ in range(nsteps):
        t = a + da
        adot_min = min(a * cos.hubble(a), t * cos.hubble(t))
        dt = O.dt_for_da(OmM, OmR, h, a, t, 1.01 * da / adot_min)
        an = O.integrate_a(OmM, OmR, h, a, dt)
        out.append((a, an, dt))
        a = an
    return out


def load_zeldovich():
    with open(os.path.join(GOLDEN, "zeldovich_pancake.json")) as f:
        return json.load(f)


def zeldovich_lattice(d, fine=False):
    """(n, stops) of the golden's 32-lattice, or of its 64-lattice when fine."""
    if fine:
        return d["lattice_fine"]["n_lattice"], d["lattice_fine"]["stops"]
    return d["n_lattice"], d["stops"]


def zeldovich_particles(d, fine=False):
    """Particles of the pancake on the golden's lattice at its first stop (z=100):
    x from the reference's perturbed_x, velocity = perturbed_v_x * a (the
    generator's proper-velocity convention), mass from the critical density."""
    P = d["params"]
    L = P["box_length"]
    n, stops = zeldovich_lattice(d, fine)
    s0 = stops[0]
    idx = np.arange(n)
    Z, Y, X = np.meshgrid(idx, idx, idx, indexing="ij")
    X, Y, Z = X.ravel(), Y.ravel(), Z.ravel()
    a0 = s0["a"]
    pos = np.stack([np.mod(np.asarray(s0["x"])[X], L), (Y + 0.5) * L / n, (Z + 0.5) * L / n], 1)
    vel = np.stack([np.asarray(s0["xdot"])[X] * a0, 0.0 * X, 0.0 * X], 1)
    h = P["H_0"] / 100.0
    mass = Cosmology(1.0, 0.0, h).rho_crit() * L ** 3 / n ** 3
    return pos, vel, mass, X, L, n, h


def zeldovich_schedule(a_from, a_to, h, rel=0.01):
    """Steps of at most 1% growth in a (nyx.relative_max_change_a = 0.01 of the
    reference run inputs) ending exactly on a_to."""
    from oracle import oracle as O
    cos = Cosmology(1.0, 0.0, h)
    out = []
    a = a_from
    while a < a_to * (1 - 1e-12):
        t = min(a * (1 + rel), a_to)
        adot_min = min(a * cos.hubble(a), t * cos.hubble(t))
        dt = O.dt_for_da(1.0, 0.0, h, a, t, 1.01 * (t - a) / adot_min)
        an = O.integrate_a(1.0, 0.0, h, a, dt)
        out.append((a, an, dt))
        a = an
    return out


def zeldovich_errors(pos, vel, stop, X, L, a):
    """Max position error / displacement amplitude, max velocity error / max velocity."""
    xa = np.asarray(stop["x"])
    amp = np.max(np.abs(xa - (np.arange(len(xa)) + 0.5) * L / len(xa)))
    dx = min_image(pos[:, 0] - np.mod(xa[X], L), L)
    va = np.asarray(stop["xdot"])[X] * a
    ex = float(np.abs(dx).max() / amp)
    ev = float(np.abs(vel[:, 0] - va).max() / np.abs(va).max())
    return ex, ev
