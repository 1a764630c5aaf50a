"""The reference's own particle input files, read from the Nyx source tree that
NYX_REFERENCE names (skipped without it):

* Exec/LyA/32.nyx, the BinaryFile IC of Exec/LyA/inputs_nohydro.rt (32^3
  particles in an 8 Mpc box at z = 100).  It holds float64 records, and the
  reader must tell that from the file size.
* Exec/ParticleOnlyTest/particle_file.2line and particle_file.mass, the
  AsciiFile inputs of that test.

Each file is parsed independently here with numpy and compared with the
library's reader bit for bit.  Then the oracle runs the DM-only step of
inputs_nohydro.rt on 32.nyx, as a realistic-input check of deposit mass and
momentum conservation (no GPU).
"""
from __future__ import annotations

import math
import os

import numpy as np
import pytest

from nyx_gb300.pm import read_particle_file, uniform_mass
from oracle import oracle as O

from tests.conftest import reference_file

LYA_IC = reference_file("Exec", "LyA", "32.nyx")
POT = os.path.dirname(reference_file("Exec", "ParticleOnlyTest", "particle_file.mass") or "")

needs_ref = pytest.mark.skipif(LYA_IC is None or not POT,
                               reason="NYX_REFERENCE (the Nyx source tree) not set")


def numpy_binary(path):
    raw = open(path, "rb").read()
    npart = int(np.frombuffer(raw[:8], dtype=np.int64)[0])
    dm, nx = (int(v) for v in np.frombuffer(raw[8:16], dtype=np.int32))
    width = (len(raw) - 16) // (npart * (dm + nx))
    rec = np.frombuffer(raw[16:], dtype=np.float64 if width == 8 else np.float32)
    rec = rec.reshape(npart, dm + nx).astype(np.float64)
    return rec[:, 0:3], rec[:, 4:7], rec[:, 3]


@needs_ref
def test_reference_binary_ic_file():
    pos, vel, mass = read_particle_file(LYA_IC, "binary")
    npos, nvel, nmass = numpy_binary(LYA_IC)
    assert len(pos) == 32 ** 3
    assert np.array_equal(pos, npos) and np.array_equal(vel, nvel) and np.array_equal(mass, nmass)
    assert pos.min() >= 0.0 and pos.max() < 8.0         # geometry.prob_hi = 8 (inputs.rt)
    assert isinstance(uniform_mass(mass), float)        # one particle mass


@needs_ref
@pytest.mark.parametrize("name,count", [("particle_file.2line", 16), ("particle_file.mass", 8)])
def test_reference_ascii_particle_files(name, count):
    path = os.path.join(POT, name)
    pos, vel, mass = read_particle_file(path, "ascii")
    rows = np.loadtxt(path, skiprows=1).reshape(-1, 7)
    assert len(pos) == count == len(rows)
    assert np.array_equal(pos, rows[:, 0:3]) and np.array_equal(mass, rows[:, 3])
    assert np.array_equal(vel, rows[:, 4:7])


@needs_ref
def test_oracle_step_on_the_reference_ics():
    """inputs_nohydro.rt: 32^3 cells, prob_hi 8, OmM 0.27, h 0.71, initial_z 100."""
    n, L, OmM, h = 32, 8.0, 0.27, 0.71
    pos, vel, mass = read_particle_file(LYA_IC, "binary")
    m = uniform_mass(mass)
    p = O.Particles(pos, vel, m)
    cs = O.sort(n, L, p)
    rho = O.deposit(n, L, p, cs)
    total = m * len(pos)
    assert rho.sum() * (L / n) ** 3 == pytest.approx(total, rel=1e-13)
    a0 = 1.0 / 101.0
    a1 = a0 * 1.01
    window = 2.0 * 0.01 * a0 / (a0 * 100 * h * math.sqrt(OmM / a0 ** 3 + (1 - OmM)))
    dt = O.dt_for_da(OmM, 0.0, h, a0, a1, window)
    a1 = O.integrate_a(OmM, 0.0, h, a0, dt)
    pm = O.PMOracle(n, L, p, OmM=OmM, OmR=0.0, h=h)
    mom0 = vel.sum(axis=0) * a0
    pm.step(a0, a1, dt)
    assert pm.cycles[0] > 0 and pm.cycles[1] > 0
    _, v1 = p.by_id()
    scale = np.abs(v1).sum() * a1
    assert np.abs(v1.sum(axis=0) * a1 - mom0).max() < 1e-9 * scale
