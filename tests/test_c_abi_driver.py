"""The C ABI used from C++ the way a Nyx-side shim would use it.

tests/c_abi/pm_driver.cpp includes include/nyxpm.h and links
nyx_gb300/libnyxpm.so with nothing else.  It reads an AsciiFile and takes PM
steps with dt from nyxpm_compute_new_dt, then writes the particles back.  On CPU
the program must compile and link.  On the GPU its result must equal the Python
(ctypes) path's, which the parity tests tie to the oracle, bit for bit.
"""
from __future__ import annotations

import os
import shutil
import subprocess

import numpy as np
import pytest

from nyx_gb300 import _lib
from nyx_gb300.pm import Box, read_particle_file, write_particle_file
from tests.conftest import gpu_available
from tests.pm_cases import config1_ics

REPO = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def build_driver(out_dir):
    _lib.load()   # builds the library if needed
    exe = os.path.join(out_dir, "pm_driver")
    libdir = os.path.join(REPO, "nyx_gb300")
    cmd = ["g++", "-O2", "-std=c++17", os.path.join(REPO, "tests", "c_abi", "pm_driver.cpp"),
           "-I", os.path.join(REPO, "include"), "-L", libdir, "-lnyxpm", f"-Wl,-rpath,{libdir}",
           "-o", exe]
    r = subprocess.run(cmd, capture_output=True, text=True)
    assert r.returncode == 0, r.stderr
    return exe


@pytest.mark.skipif(shutil.which("g++") is None, reason="no C++ compiler")
def test_driver_compiles_and_links_against_the_header_alone(tmp_path):
    exe = build_driver(str(tmp_path))
    r = subprocess.run([exe], capture_output=True, text=True)
    assert r.returncode == 2 and "usage" in r.stderr


@pytest.mark.gpu
@pytest.mark.skipif(not gpu_available(), reason="no GPU")
def test_driver_result_equals_python_path(ctx, tmp_path):
    exe = build_driver(str(tmp_path))
    n = 32
    ic = config1_ics(n, seed=8)
    inp, out = str(tmp_path / "in.ascii"), str(tmp_path / "out.ascii")
    write_particle_file(inp, ic.pos, ic.vel, ic.mass)
    r = subprocess.run([exe, inp, str(n), "1.0", "0.02", "4", out], capture_output=True, text=True)
    assert r.returncode == 0, r.stderr
    cpos, cvel, _ = read_particle_file(out)
    pos, vel, _ = read_particle_file(inp)
    box = Box(ctx, n, 1.0, len(pos))
    box.upload(pos, vel, ic.mass)
    box.init_field(0.02)
    t, a, dt_old = 0.0, 0.02, -1.0
    for line in r.stdout.strip().splitlines():
        dt, a_new = box.compute_new_dt(t, a, dt_old)
        assert f"a {a_new:.17g} dt {dt:.17g}" in line
        box.step(a, a_new, dt)
        t, a, dt_old = t + dt, a_new, dt
    ppos, pvel = box.download()
    assert np.array_equal(cpos, ppos) and np.array_equal(cvel, pvel)
    box.close()


@pytest.mark.gpu
@pytest.mark.skipif(not gpu_available(), reason="no GPU")
def test_driver_kicks_with_the_callers_acceleration(tmp_path):
    """moveKickDrift with a caller-owned acc (DarkMatterParticleContainer.cpp:76-112):
    the C++ caller hands the oracle's gravity vector over with nyxpm_set_grav_vector
    and kicks; the result equals the oracle's update_dm_particle_single bit for bit."""
    from oracle import oracle as O
    exe = build_driver(str(tmp_path))
    n, L = 16, 1.0
    ic = config1_ics(n, seed=12)
    rng = np.random.default_rng(3)
    g = rng.standard_normal(3 * n ** 3) * 50.0
    inp, out = str(tmp_path / "in.ascii"), str(tmp_path / "out.ascii")
    accf = str(tmp_path / "acc.f64")
    write_particle_file(inp, ic.pos, ic.vel, ic.mass)
    g.astype("<f8").tofile(accf)
    dt, a_old, a_half = 2.0e-4, 0.031, 0.0335
    r = subprocess.run([exe, "kick", inp, str(n), str(L), accf, f"{dt:.17g}", f"{a_old:.17g}",
                        f"{a_half:.17g}", out], capture_output=True, text=True)
    assert r.returncode == 0, r.stderr
    cpos, cvel, _ = read_particle_file(out)
    pos, vel, _ = read_particle_file(inp)
    p = O.Particles(pos, vel, ic.mass)
    O.move(n, L, p, g, dt, a_old, a_half, 1)
    opos, ovel = p.by_id()
    assert np.array_equal(cpos, opos) and np.array_equal(cvel, ovel)


@pytest.mark.gpu
@pytest.mark.skipif(not gpu_available(), reason="no GPU")
def test_driver_runs_the_reference_multilevel_test(tmp_path):
    """The reference's Exec/ParticleOnlyTest/inputs.mass.nosub setup through the C
    ABI from C++: its AsciiFile particles on its fixed grids (amr.regrid_file), no
    subcycling, a = 1; three multilevel steps against the multilevel oracle
    (positions 1e-13, velocity change 1e-8: the GPU deposit adds with atomics)."""
    from nyx_gb300.amr import regrid_file_boxes
    from oracle import oracle as O
    exe = build_driver(str(tmp_path))
    golden = os.path.join(REPO, "tests", "golden")
    with open(os.path.join(golden, "particle_only_fixed_grids.mass")) as f:
        boxes = regrid_file_boxes(f)
    inp = os.path.join(golden, "particle_only_particle_file.mass")
    out = str(tmp_path / "out.ascii")
    args = [exe, "amr", inp, "16", "32.0", "1.0", "0.05", "3", out, str(len(boxes) + 1)]
    args += [str(len(lv)) for lv in boxes]
    args += [str(v) for lv in boxes for lo, hi in lv for v in (*lo, *hi)]
    r = subprocess.run(args, capture_output=True, text=True)
    assert r.returncode == 0, r.stderr
    assert len(r.stdout.strip().splitlines()) == 3
    cpos, cvel, _ = read_particle_file(out)
    pos, vel, mass = read_particle_file(inp)
    p = O.Particles(pos, vel, mass)
    A = O.AmrOracle(16, 32.0, boxes, p)
    for _ in range(3):
        assert A.step(1.0, 1.0, 0.05) == 0
    rel = lambda a, b: float(np.linalg.norm(a - b) / np.linalg.norm(b))
    assert rel(cpos, p.pos()) <= 1e-13
    assert rel(cvel - vel, p.vel() - vel) <= 1e-8
