"""Nyx inputs files (AMReX ParmParse syntax) for the particle-only PM run.

A Nyx inputs file holds one ``key = value value ...`` per line; ``#`` starts a
comment, values may be double-quoted, and a later assignment overrides an
earlier one.  ``run_config`` takes the keys a dark-matter-only, single-level,
periodic run uses (names and defaults as Nyx reads them:
Source/Driver/Nyx.cpp:278-449, Source/Driver/comoving.cpp:16-72,
Source/Particle/NyxParticles.cpp:262-376, Source/Gravity/Gravity.cpp:76-114)
and refuses inputs outside that scope (hydro, AMR levels, non-periodic or
non-cubic domains) with a clear message.
"""
from __future__ import annotations

import os
import shlex
from dataclasses import dataclass


def read_inputs(path: str, overrides: list[str] | None = None) -> dict[str, list[str]]:
    """key -> list of value tokens; ``overrides`` are extra "key=value" items (the
    command-line form), applied last."""
    out: dict[str, list[str]] = {}
    with open(path) as f:
        lines = f.read().splitlines()
    for line in lines + list(overrides or []):
        line = line.split("#", 1)[0].strip()
        if not line or "=" not in line:
            continue
        key, val = line.split("=", 1)
        key = key.strip()
        if key:
            out[key] = shlex.split(val)
    return out


def _str(d, key, default):
    vals = d.get(key)
    return vals[0] if vals else default


def _get(d, key, default, conv=float, n=1):
    if key not in d:
        return default
    vals = [conv(v) for v in d[key]]
    return vals[0] if n == 1 else vals


@dataclass
class RunConfig:
    n: int
    L: float
    OmM: float
    OmB: float
    h: float
    initial_z: float
    final_a: float             # -1: no final a
    stop_time: float           # -1: none
    max_step: int
    rel_tol: float
    cfl: float
    change_max: float
    init_shrink: float
    relative_max_change_a: float
    absolute_max_change_a: float
    dt_binpow: float
    dt_cutoff: float
    particle_file: str         # the particle file, cosmo.initDirName for "cosmological",
                               # <restart_particle_file>/DM for "restart"
    particle_format: str       # ascii | binary | binary_meta | cosmological | restart
    ic_source: str             # cosmo.ic-source (MUSIC | nyx) for "cosmological"
    n_particles: int           # nyx.n_particles per edge (the nyx source's particle mass)
    plot_int: int
    plot_file: str
    check_int: int
    check_file: str
    data_log: str
    restart: str
    ascii_output: bool = False  # particles.dm_particle_output_ascii: plotfiles add particles.ascii


def run_config(d: dict[str, list[str]], base_dir: str = ".") -> RunConfig:
    """The particle-only run an inputs dict describes; ValueError outside the scope."""
    if _get(d, "nyx.do_hydro", 1, int) != 0:
        raise ValueError("nyx.do_hydro must be 0: the GPU step is dark matter only")
    if _get(d, "amr.max_level", 0, int) != 0:
        raise ValueError("amr.max_level must be 0: the GPU step is single-level")
    if _get(d, "nyx.do_grav", 1, int) != 1 or _get(d, "nyx.do_dm_particles", 1, int) != 1:
        raise ValueError("nyx.do_grav and nyx.do_dm_particles must be 1")
    per = _get(d, "geometry.is_periodic", [1, 1, 1], int, 3)
    if list(per) != [1, 1, 1]:
        raise ValueError("geometry.is_periodic must be 1 1 1")
    ncell = _get(d, "amr.n_cell", None, int, 3)
    if ncell is None or len(set(ncell)) != 1:
        raise ValueError("amr.n_cell must give one cubic grid, e.g. 64 64 64")
    lo = _get(d, "geometry.prob_lo", [0.0, 0.0, 0.0], float, 3)
    hi = _get(d, "geometry.prob_hi", None, float, 3)
    if hi is None:
        raise ValueError("geometry.prob_hi is required")
    sides = [h - l for l, h in zip(lo, hi)]
    if any(abs(s - sides[0]) > 1e-12 * sides[0] for s in sides) or any(v != 0.0 for v in lo):
        raise ValueError("the domain must be a cube with geometry.prob_lo = 0 0 0")
    init = _str(d, "nyx.particle_init_type", "AsciiFile")
    fmt = {"AsciiFile": "ascii", "BinaryFile": "binary", "BinaryMetaFile": "binary_meta",
           "Cosmological": "cosmological", "Restart": "restart"}.get(init)
    if fmt is None:
        raise ValueError(f"nyx.particle_init_type {init} is not supported "
                         "(AsciiFile, BinaryFile, BinaryMetaFile, Cosmological, Restart)")
    ic_source, n_part = "", ncell[0]
    if fmt == "cosmological":
        # Nyx::initcosmo (Source/Initialization/Nyx_initcosmo.cpp:100-427): the IC
        # MultiFab <cosmo.initDirName>/Level_0/Cell, one particle per cell
        key = "cosmo.initDirName"
        ic_source = _str(d, "cosmo.ic-source", "")
        if ic_source not in ("MUSIC", "nyx"):
            raise ValueError("cosmo.ic-source must be MUSIC or nyx for particle_init_type Cosmological")
        if _get(d, "nyx.initial_z", None) is None:
            raise ValueError("nyx.initial_z is required for particle_init_type Cosmological")
        npv = _get(d, "nyx.n_particles", None, int, 3)
        if npv is None and ic_source == "nyx":
            raise ValueError("nyx.n_particles is required for cosmo.ic-source nyx")
        if npv is not None:
            if len(set(npv)) != 1:
                raise ValueError("nyx.n_particles must be the same on each axis")
            n_part = npv[0]
    elif fmt == "restart":
        # the DM directory of a plotfile or checkpoint (NyxParticles.cpp:584-586)
        key = "nyx.restart_particle_file"
    else:
        key = "nyx.ascii_particle_file" if fmt == "ascii" else "nyx.binary_particle_file"
    pfile = _str(d, key, "")
    if not pfile:
        raise ValueError(f"{key} is required for particle_init_type {init}")
    if not os.path.isabs(pfile):
        pfile = os.path.join(base_dir, pfile)
    if fmt == "restart":
        pfile = os.path.join(pfile, "DM")
    final_a = _get(d, "nyx.final_a", -1.0)
    final_z = _get(d, "nyx.final_z", -1.0)
    if final_a <= 0 and final_z >= 0:
        final_a = 1.0 / (1.0 + final_z)
    return RunConfig(
        n=ncell[0], L=sides[0],
        OmM=_get(d, "nyx.comoving_OmM", 1.0), OmB=_get(d, "nyx.comoving_OmB", 0.0),
        h=_get(d, "nyx.comoving_h", 0.0),
        initial_z=_get(d, "nyx.initial_z", -1.0), final_a=final_a,
        stop_time=_get(d, "stop_time", -1.0), max_step=_get(d, "max_step", 2 ** 31 - 1, int),
        rel_tol=_get(d, "gravity.sl_tol", 1e-12), cfl=_get(d, "particles.cfl", 0.5),
        change_max=_get(d, "nyx.change_max", 1.1), init_shrink=_get(d, "nyx.init_shrink", 1.0),
        relative_max_change_a=_get(d, "nyx.relative_max_change_a", 0.01),
        absolute_max_change_a=_get(d, "nyx.absolute_max_change_a", -1.0),
        dt_binpow=_get(d, "nyx.dt_binpow", -1.0), dt_cutoff=_get(d, "nyx.dt_cutoff", 0.0),
        particle_file=pfile, particle_format=fmt, ic_source=ic_source, n_particles=n_part,
        plot_int=_get(d, "amr.plot_int", -1, int), plot_file=_str(d, "amr.plot_file", "plt"),
        check_int=_get(d, "amr.check_int", -1, int), check_file=_str(d, "amr.check_file", "chk"),
        data_log=_str(d, "amr.data_log", ""), restart=_str(d, "amr.restart", ""),
        ascii_output=_get(d, "particles.dm_particle_output_ascii", 0, int) != 0)
