"""The Nyx-style run driver (python -m nyx_gb300.run) on the GPU.

* a run from an inputs file takes the same steps as the library calls made by
  hand (computeInitialDt / computeNewDt, then the PM step), bit for bit;
* restarting from a checkpoint directory gives the uninterrupted result bit
  for bit;
* the runlog and the plot/checkpoint directories are written.
"""
from __future__ import annotations

import os

import numpy as np
import pytest

from nyx_gb300.pm import (Box, particles_info, read_comoving_a, read_particles_dir,
                          write_particle_file)
from nyx_gb300.run import run
from tests.pm_cases import config1_ics

pytestmark = pytest.mark.gpu


def write_inputs(tmp_path, extra=""):
    ic = config1_ics(16, seed=12, a_init=0.05)
    write_particle_file(tmp_path / "ics.ascii", ic.pos, ic.vel, ic.mass)
    text = ("max_step = 6\n"
            "nyx.initial_z = 19.0\n"          # a = 0.05
            "nyx.final_z = 0.0\n"
            "geometry.is_periodic = 1 1 1\n"
            "geometry.prob_lo = 0 0 0\n"
            "geometry.prob_hi = 1.0 1.0 1.0\n"
            "amr.n_cell = 16 16 16\n"
            "amr.max_level = 0\n"
            "nyx.do_hydro = 0\n"
            "nyx.comoving_OmM = 1.0\n"
            "nyx.comoving_h = 0.675\n"
            "nyx.particle_init_type = AsciiFile\n"
            "nyx.ascii_particle_file = ics.ascii\n"
            "gravity.sl_tol = 1.e-10\n"
            "nyx.relative_max_change_a = 0.01\n"
            "particles.cfl = 0.5\n"
            "nyx.init_shrink = 0.5\n"
            "amr.data_log = runlog\n"
            "amr.plot_int = 2\n"
            "amr.check_int = 3\n" + extra)
    p = tmp_path / "inputs"
    p.write_text(text)
    return str(p), ic


def test_run_matches_the_library_calls_and_restarts_exactly(ctx, tmp_path):
    inp, ic = write_inputs(tmp_path)
    res = run(inp, out_dir=str(tmp_path), verbose=False)
    assert res["steps"] == 6 and res["last_step"] == 6
    # the same steps by hand
    box = Box(ctx, 16, 1.0, len(ic.pos))
    box.upload(ic.pos, ic.vel, ic.mass)
    a, t, dt_old = 0.05, 0.0, -1.0
    box.init_field(a)
    for s in range(6):
        dt, a_new = box.compute_new_dt(t, a, dt_old, cfl=0.5, relative_max_change_a=0.01, final_a=1.0)
        if s == 0:
            dt = dt * 0.5
            a_new = ctx.integrate_comoving_a(a, dt)
        box.step(a, a_new, dt)
        t, a, dt_old = t + dt, a_new, dt
    pos, vel = box.download()
    box.close()
    assert np.array_equal(pos, res["pos"]) and np.array_equal(vel, res["vel"])
    assert res["a"] == a
    # outputs
    log = (tmp_path / "runlog").read_text().splitlines()
    assert len(log) == 7 and log[0].startswith("#")
    for d in ("plt00002", "plt00004", "plt00006", "chk00003", "chk00006"):
        assert (tmp_path / d / "comoving_a").exists(), d
        assert (tmp_path / d / "DM" / "Header").exists(), d
    # the checkpoint's DM directory holds the particles of step 3 with their ids
    assert particles_info(str(tmp_path / "chk00003" / "DM"))["is_checkpoint"] == 1
    assert particles_info(str(tmp_path / "plt00006" / "DM"))["is_checkpoint"] == 0
    ppos, pvel, _ = read_particles_dir(str(tmp_path / "plt00006" / "DM"))
    assert np.array_equal(ppos, res["pos"]) and np.array_equal(pvel, res["vel"])
    assert abs(read_comoving_a(str(tmp_path / "chk00006")) - a) <= 1e-14 * a
    assert (tmp_path / "chk00003" / "phi.f64").stat().st_size == 8 * 16 ** 3
    # restart from step 3 and finish: the uninterrupted result, bit for bit
    out2 = tmp_path / "restart"
    out2.mkdir()
    res2 = run(inp, ["amr.restart=" + str(tmp_path / "chk00003"), "amr.data_log="],
               out_dir=str(out2), verbose=False)
    assert res2["steps"] == 3 and res2["last_step"] == 6
    assert np.array_equal(res2["pos"], res["pos"]) and np.array_equal(res2["vel"], res["vel"])
    # a run that starts from the plotfile's particles (nyx.particle_init_type = Restart)
    res3 = run(inp, ["nyx.particle_init_type=Restart", "nyx.restart_particle_file=plt00006",
                     "max_step=1", "amr.data_log=", "amr.plot_int=-1", "amr.check_int=-1"],
               out_dir=str(tmp_path), verbose=False)
    assert res3["steps"] == 1 and res3["particles"] == len(res["pos"])


def test_mixed_precision_run(tmp_path):
    inp, ic = write_inputs(tmp_path, "amr.plot_int = -1\namr.check_int = -1\n")
    fp = run(inp, out_dir=str(tmp_path), verbose=False)
    mx = run(inp, ["amr.data_log="], precision="mixed", out_dir=str(tmp_path), verbose=False)
    disp = np.linalg.norm((fp["pos"] - ic.pos + 0.5) % 1.0 - 0.5)
    err = np.linalg.norm((mx["pos"] - fp["pos"] + 0.5) % 1.0 - 0.5)
    assert err <= 1e-5 * disp


@pytest.mark.parametrize("source", ["MUSIC", "nyx"])
def test_run_from_an_ic_multifab(ctx, tmp_path, source):
    """particle_init_type = Cosmological: one particle per cell from the IC
    MultiFab <cosmo.initDirName>/Level_0/Cell with Nyx::initcosmo's factors and
    mass; the run equals the same fields placed by hand with init_cosmo_1ppc."""
    from nyx_gb300 import multifab as M
    n = 16
    ic = config1_ics(n, seed=13, a_init=0.05)
    disp = ((ic.pos - ic.lattice + 0.5) % 1.0 - 0.5).T.reshape(3, n, n, n)
    vel = ic.vel.T.reshape(3, n, n, n)
    fields = np.concatenate([disp, vel * 1e-3]) if source == "MUSIC" else disp
    M.write(M.ic_multifab_name(str(tmp_path / "ics_mf")), fields, max_grid_size=8)
    inp, _ = write_inputs(tmp_path, "amr.plot_int = -1\namr.check_int = -1\nmax_step = 3\n"
                                    "nyx.particle_init_type = Cosmological\n"
                                    "cosmo.initDirName = ics_mf\n"
                                    f"cosmo.ic-source = {source}\n"
                                    "nyx.n_particles = 16 16 16\n")
    res = run(inp, ["amr.data_log="], out_dir=str(tmp_path), verbose=False)
    assert res["steps"] == 3 and res["particles"] == n ** 3
    d_ic, v_ic = M.read_ic_fields(str(tmp_path / "ics_mf"), source, n)
    dfac, vfac, pmass = ctx.cosmo_ic_factors(source, n, 1.0, 19.0)
    box = Box(ctx, n, 1.0, n ** 3)
    box.init_cosmo_1ppc(d_ic, v_ic, dfac, vfac, pmass)
    a, t, dt_old = 0.05, 0.0, -1.0
    box.init_field(a)
    for s in range(3):
        dt, a_new = box.compute_new_dt(t, a, dt_old, cfl=0.5, relative_max_change_a=0.01, final_a=1.0)
        if s == 0:
            dt = dt * 0.5
            a_new = ctx.integrate_comoving_a(a, dt)
        box.step(a, a_new, dt)
        t, a, dt_old = t + dt, a_new, dt
    pos, v = box.download()
    box.close()
    assert np.array_equal(pos, res["pos"]) and np.array_equal(v, res["vel"])
