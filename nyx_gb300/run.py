"""A Nyx-style particle-only run on one GPU, driven by a Nyx inputs file.

    python -m nyx_gb300.run <inputs> [key=value ...] [--precision mixed]

What it does, following Nyx's driver on one periodic level:
1. It reads the particles named by ``nyx.particle_init_type``: a particle file,
   or (Cosmological) one particle per cell from the IC MultiFab
   ``<cosmo.initDirName>/Level_0/Cell`` as Nyx::initcosmo places them.
2. It solves for the initial field at a = 1 / (1 + nyx.initial_z), as
   Nyx::post_init does.
3. It takes PM steps, ``Nyx::advance_particles_only`` plus ``post_timestep``.
   The first dt is ``computeInitialDt`` (init_shrink x the estimate).  Later ones
   are ``computeNewDt``: particle CFL, the a-change limits, change_max,
   stop_time and final_a.
4. It stops at max_step, at stop_time, at final_a or when dt falls below
   nyx.dt_cutoff.

Output:
- ``amr.data_log``: the runlog, one line of nstep, time, dt, z, a per step
  (Source/IO/write_info.cpp:46-60).
- ``amr.plot_file`` directories every ``amr.plot_int`` steps: the particles in
  ``DM/`` as Nyx's plotfile writes them (the AMReX particle layout
  Version_Two_Dot_Zero, float64, no ids, with the ``precision`` file of
  Source/IO/Nyx_output.cpp:677-688), ``particles.ascii`` when
  ``particles.dm_particle_output_ascii = 1``, and the ``comoving_a`` file.
- ``amr.check_file`` directories every ``amr.check_int`` steps: the particles in
  ``DM/`` as Nyx's checkpoint writes them (the same layout with ids, float64:
  a Nyx restart with ``nyx.particle_init_type = Restart`` reads them), the
  potential (``phi.f64``), ``comoving_a`` and the exact step, time, dt and a.
  ``amr.restart = <dir>`` resumes from one bit for bit (FP64 path).
- ``nyx.particle_init_type = Restart`` starts from the ``DM/`` particles of a
  Nyx plotfile or checkpoint named by ``nyx.restart_particle_file``.
"""
from __future__ import annotations

import argparse
import json
import os
import sys
import time

import numpy as np

from . import inputs as _inputs
from .multifab import read_ic_fields
from .pm import (Box, Context, read_comoving_a, read_particle_file, read_particles_dir,
                 uniform_mass, write_comoving_a, write_particle_file, write_particles_dir)

STATE_FILE = "run_state.json"
PHI_FILE = "phi.f64"            # PhiGrav_Type, n^3 float64, x fastest


def _write_dir(path, box, step, t, dt, a, exact, ascii_output=False):
    os.makedirs(path, exist_ok=True)
    pos, vel = box.download()
    # the DM directory as Nyx writes it (particle_check_point / particle_plot_file)
    write_particles_dir(os.path.join(path, "DM"), box.n, pos, vel, box.mass, checkpoint=exact)
    if exact:
        box.get_phi().tofile(os.path.join(path, PHI_FILE))
        with open(os.path.join(path, STATE_FILE), "w") as f:
            json.dump({"step": step, "time": t.hex(), "dt": dt.hex(), "a": a.hex()}, f)
    else:
        with open(os.path.join(path, "DM", "precision"), "w") as f:
            f.write("NATIVE\n")
        if ascii_output:
            write_particle_file(os.path.join(path, "particles.ascii"), pos, vel, box.mass, "ascii")
    write_comoving_a(path, a)


def run(inputs_path: str, overrides: list[str] | None = None, precision: str = "fp64",
        out_dir: str | None = None, verbose: bool = True, device: int = 0) -> dict:
    base = os.path.dirname(os.path.abspath(inputs_path))
    cfg = _inputs.run_config(_inputs.read_inputs(inputs_path, overrides), base)
    out_dir = out_dir or os.getcwd()
    ctx = Context(device=device, OmM=cfg.OmM, OmR=0.0, h=cfg.h, rel_tol=cfg.rel_tol)
    dtp = dict(cfl=cfg.cfl, change_max=cfg.change_max,
               relative_max_change_a=cfg.relative_max_change_a,
               absolute_max_change_a=cfg.absolute_max_change_a, final_a=cfg.final_a,
               stop_time=cfg.stop_time, dt_binpow=cfg.dt_binpow)
    if cfg.restart:
        rdir = cfg.restart if os.path.isabs(cfg.restart) else os.path.join(out_dir, cfg.restart)
        with open(os.path.join(rdir, STATE_FILE)) as f:
            st = json.load(f)
        step, t, dt_old, a = (st["step"], float.fromhex(st["time"]), float.fromhex(st["dt"]),
                              float.fromhex(st["a"]))
        pos, vel, mass = read_particles_dir(os.path.join(rdir, "DM"))
        if abs(read_comoving_a(rdir) - a) > 1e-14 * a:
            raise ValueError(f"{rdir}: comoving_a does not match the run state")
    else:
        step, t, dt_old = 0, 0.0, -1.0
        a = 1.0 / (1.0 + cfg.initial_z)
        if cfg.particle_format == "restart":
            pos, vel, mass = read_particles_dir(cfg.particle_file)
        elif cfg.particle_format != "cosmological":
            pos, vel, mass = read_particle_file(cfg.particle_file, cfg.particle_format)
    if not cfg.restart and cfg.particle_format == "cosmological":
        disp, ivel = read_ic_fields(cfg.particle_file, cfg.ic_source, cfg.n)
        # MUSIC: mass rho_m dx^3 of the grid; nyx: rho_m L^3 / n_particles^3
        n_mass = cfg.n_particles if cfg.ic_source == "nyx" else cfg.n
        dfac, vfac, pmass = ctx.cosmo_ic_factors(cfg.ic_source, n_mass, cfg.L, cfg.initial_z)
        box = Box(ctx, cfg.n, cfg.L, cfg.n ** 3, precision=precision)
        box.init_cosmo_1ppc(disp, ivel, dfac, vfac, pmass)
    else:
        box = Box(ctx, cfg.n, cfg.L, len(pos), precision=precision)
        box.upload(pos, vel, uniform_mass(mass))
    if cfg.restart:
        # the checkpointed field, as Nyx restores PhiGrav_Type: the next dt
        # estimate then sees the same gravity as the uninterrupted run
        box.set_phi(np.fromfile(os.path.join(rdir, PHI_FILE), dtype=np.float64))
    else:
        box.init_field(a)
    log = open(os.path.join(out_dir, cfg.data_log), "a") if cfg.data_log else None
    if log and step == 0:
        log.write(f"{'#  nstep':>8}{'time':>24}{'dt':>24}{'z':>24}{'a':>24}\n")
    t0 = time.perf_counter()
    steps_done = 0
    while step < cfg.max_step:
        if cfg.final_a > 0 and a >= cfg.final_a * (1 - 1e-12):
            break
        if cfg.stop_time >= 0 and t >= cfg.stop_time * (1 - 1e-12):
            break
        dt, a_new = box.compute_new_dt(t, a, dt_old, **dtp)
        if dt_old <= 0 and cfg.init_shrink != 1.0:         # computeInitialDt
            dt = dt * cfg.init_shrink
            a_new = ctx.integrate_comoving_a(a, dt)
        if dt < cfg.dt_cutoff:
            if verbose:
                print(f"dt {dt:.3e} below nyx.dt_cutoff: stopping", file=sys.stderr)
            break
        box.step(a, a_new, dt)
        step += 1
        steps_done += 1
        t, a, dt_old = t + dt, a_new, dt
        if log:
            log.write(f"{step:8d}{t:24.16e}{dt:24.16e}{1.0 / a - 1.0:24.16e}{a:24.16e}\n")
        if verbose:
            print(f"step {step:6d}  a {a:.8f}  z {1.0 / a - 1.0:9.4f}  dt {dt:.4e}", file=sys.stderr)
        if cfg.plot_int > 0 and step % cfg.plot_int == 0:
            _write_dir(os.path.join(out_dir, f"{cfg.plot_file}{step:05d}"), box, step, t, dt, a, False,
                       cfg.ascii_output)
        if cfg.check_int > 0 and step % cfg.check_int == 0:
            _write_dir(os.path.join(out_dir, f"{cfg.check_file}{step:05d}"), box, step, t, dt, a, True)
    wall = time.perf_counter() - t0
    if log:
        log.close()
    pos, vel = box.download()
    box.close()
    ctx.close()
    return {"steps": steps_done, "last_step": step, "time": t, "a": a, "z": 1.0 / a - 1.0,
            "wall_s": wall, "particles": len(pos),
            "particle_steps_per_s": len(pos) * steps_done / wall if wall > 0 else 0.0,
            "pos": pos, "vel": vel}


def main(argv=None):
    ap = argparse.ArgumentParser(description=__doc__.split("\n\n")[0])
    ap.add_argument("inputs")
    ap.add_argument("overrides", nargs="*", help="key=value items applied after the file")
    ap.add_argument("--precision", choices=["fp64", "mixed"], default="fp64")
    ap.add_argument("--out", default=None, help="directory for the runlog and output (cwd)")
    a = ap.parse_args(argv)
    res = run(a.inputs, a.overrides, a.precision, a.out)
    print(json.dumps({k: v for k, v in res.items() if k not in ("pos", "vel")}))
    return 0


if __name__ == "__main__":
    sys.exit(main())
