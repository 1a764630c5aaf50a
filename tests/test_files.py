"""Nyx's particle initial-condition files and the comoving_a file, read and
written by the library's host code (no GPU).

Formats (Docs/sphinx_documentation/source/ICs.rst:13-78): AsciiFile (count line,
then "x y z mass vx vy vz"), BinaryFile (int64 NP, int32 DM = 3, int32 NX >= 4,
then NP records of DM + NX float32), BinaryMetaFile (a list of binary files).
The test files are written here with numpy, independently of the library.
"""
from __future__ import annotations

import numpy as np
import pytest

from nyx_gb300.pm import (NyxPMError, read_comoving_a, read_particle_file, uniform_mass,
                          write_comoving_a, write_particle_file)


def particles(n=1000, seed=3):
    rng = np.random.default_rng(seed)
    return rng.random((n, 3)), rng.standard_normal((n, 3)) * 300.0, rng.random(n) * 1e10 + 1e9


def write_binary(path, pos, vel, mass, nx=4):
    rec = np.zeros((len(pos), 3 + nx), dtype=np.float32)
    rec[:, 0:3] = pos
    rec[:, 3] = mass
    rec[:, 4:7] = vel
    if nx > 4:
        rec[:, 7:] = -1.0
    with open(path, "wb") as f:
        f.write(np.int64(len(pos)).tobytes())
        f.write(np.int32(3).tobytes())
        f.write(np.int32(nx).tobytes())
        f.write(rec.tobytes())


def test_ascii_file_reads_exactly(tmp_path):
    pos, vel, mass = particles()
    p = tmp_path / "ics.ascii"
    with open(p, "w") as f:
        f.write(f"{len(pos)}\n")
        for q in range(len(pos)):
            f.write(" ".join(repr(float(v)) for v in (*pos[q], mass[q], *vel[q])) + "\n")
    rp, rv, rm = read_particle_file(p, "ascii")
    assert np.array_equal(rp, pos) and np.array_equal(rv, vel) and np.array_equal(rm, mass)


@pytest.mark.parametrize("nx", [4, 6])
def test_binary_file_reads_float32_records(tmp_path, nx):
    pos, vel, mass = particles(777)
    p = tmp_path / "ics.bin"
    write_binary(p, pos, vel, mass, nx)
    rp, rv, rm = read_particle_file(p, "binary")
    assert np.array_equal(rp, pos.astype(np.float32).astype(np.float64))
    assert np.array_equal(rv, vel.astype(np.float32).astype(np.float64))
    assert np.array_equal(rm, mass.astype(np.float32).astype(np.float64))


def test_binary_meta_file_concatenates_in_order(tmp_path):
    parts = [particles(300, s) for s in (1, 2, 3)]
    names = []
    for i, (pos, vel, mass) in enumerate(parts):
        names.append(tmp_path / f"part{i}.bin")
        write_binary(names[-1], pos, vel, mass)
    meta = tmp_path / "ics.meta"
    meta.write_text("\n".join(str(n) for n in names) + "\n\n")
    rp, rv, rm = read_particle_file(meta, "binary_meta")
    want = np.concatenate([p[0] for p in parts]).astype(np.float32).astype(np.float64)
    assert np.array_equal(rp, want) and len(rm) == 900


@pytest.mark.parametrize("fmt", ["ascii", "binary"])
def test_write_then_read_round_trip(tmp_path, fmt):
    pos, vel, mass = particles(500)
    p = tmp_path / f"out.{fmt}"
    write_particle_file(p, pos, vel, 2.5e9, fmt)
    rp, rv, rm = read_particle_file(p, fmt)
    if fmt == "ascii":
        assert np.array_equal(rp, pos) and np.array_equal(rv, vel)
    else:
        assert np.array_equal(rp, pos.astype(np.float32))
    assert uniform_mass(rm) == 2.5e9


def test_malformed_files_are_errors(tmp_path):
    bad = tmp_path / "short.ascii"
    bad.write_text("3\n0.1 0.2 0.3 1 0 0 0\n0.1 0.2\n")
    with pytest.raises(NyxPMError, match="incomplete"):
        read_particle_file(bad, "ascii")
    hdr = tmp_path / "dm2.bin"
    with open(hdr, "wb") as f:
        f.write(np.int64(1).tobytes() + np.int32(2).tobytes() + np.int32(4).tobytes())
    with pytest.raises(NyxPMError, match="DM = 3"):
        read_particle_file(hdr, "binary")
    with pytest.raises(NyxPMError, match="cannot"):
        read_particle_file(tmp_path / "missing.bin", "binary")


def test_comoving_a_file(tmp_path):
    a = 0.0296047342259805712
    write_comoving_a(tmp_path, a)
    text = (tmp_path / "comoving_a").read_text()
    assert text == f"{a:.15g}\n"                  # File.precision(15) << a
    assert read_comoving_a(tmp_path) == float(f"{a:.15g}")


def test_cosmo_1ppc_particles_equal_oracle():
    """InitCosmo1ppcMultiLevel: cell centres plus scaled displacements, periodic
    shift (also of displacements beyond a box length), scaled velocities."""
    from nyx_gb300.pm import cosmo_1ppc_particles
    from oracle import oracle as O
    n, L = 16, 7.5
    rng = np.random.default_rng(9)
    disp = rng.standard_normal((3, n ** 3)) * 0.05
    disp[0, :10] = 1.7            # more than one box length (in units of L)
    disp[1, 10:20] = -0.999
    vel = rng.standard_normal((3, n ** 3))
    df, vf = [L, L, L], [3.1, 3.1, 3.1]
    pos, v = cosmo_1ppc_particles(n, L, disp, vel, df, vf)
    opos, ov = O.cosmo_1ppc(n, L, disp, vel, df, vf)
    assert np.array_equal(pos, opos) and np.array_equal(v, ov)
    assert pos.min() >= 0.0 and pos.max() < L


def test_cosmo_ic_factors_match_initcosmo():
    """Nyx_initcosmo.cpp:185-294 for ic-source MUSIC and nyx, dark matter only."""
    import math
    from nyx_gb300.pm import Context
    from oracle import oracle as O
    ctx = Context.__new__(Context)          # host-only: no device context needed
    import ctypes as C
    from nyx_gb300 import _lib as L
    ctx.lib = L.load()
    ctx.params = L.Params()
    ctx.lib.nyxpm_default_params(C.byref(ctx.params))
    ctx.params.comoving_OmM, ctx.params.comoving_h = 0.3, 0.7
    G = O.gconst()
    rho = 3 * 0.7 * 100 * 0.7 * 100 * 0.3 / (8 * math.pi * G)
    df, vf, m = ctx.cosmo_ic_factors("MUSIC", 64, 100.0)
    assert df == [100.0] * 3 and vf == [100.0 * 0.7] * 3
    assert m == rho * (100.0 / 64) ** 3
    df, vf, m = ctx.cosmo_ic_factors("nyx", 64, 100.0, redshift=99.0)
    a = 1 / (1 + 99.0)
    assert vf[0] == 100.0 * a * math.sqrt(0.3 / math.pow(a, 3) + (1 - 0.3)) * 0.7 * 100
    assert m == rho * (100.0 * 100.0 * 100.0) / (64.0 * 64 * 64)


def test_float64_binary_round_trip_is_exact(tmp_path):
    pos, vel, mass = particles(333, seed=5)
    p = tmp_path / "exact.bin"
    write_particle_file(p, pos, vel, mass, "binary64")
    assert p.stat().st_size == 16 + 333 * 7 * 8
    rp, rv, rm = read_particle_file(p, "binary")
    assert np.array_equal(rp, pos) and np.array_equal(rv, vel) and np.array_equal(rm, mass)
