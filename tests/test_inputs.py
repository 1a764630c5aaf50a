"""Nyx inputs files (ParmParse syntax) -> the particle-only run configuration."""
from __future__ import annotations

import os

import pytest

from nyx_gb300.inputs import read_inputs, run_config

from tests.conftest import reference_file

NOHYDRO = reference_file("Exec", "LyA", "inputs_nohydro.rt")


def test_syntax_comments_quotes_and_overrides(tmp_path):
    p = tmp_path / "inputs"
    p.write_text('amr.n_cell = 16 16 16   # grid\n'
                 '# a comment line\n'
                 'nyx.uvb_rates_file = "TREECOOL middle"\n'
                 'geometry.prob_hi = 2 2 2\n'
                 'geometry.prob_hi = 4 4 4\n')
    d = read_inputs(str(p), ["max_step=7"])
    assert d["amr.n_cell"] == ["16", "16", "16"]
    assert d["nyx.uvb_rates_file"] == ["TREECOOL middle"]
    assert d["geometry.prob_hi"] == ["4", "4", "4"]      # the later assignment wins
    assert d["max_step"] == ["7"]


def test_scope_is_enforced(tmp_path):
    base = {"amr.n_cell": ["16", "16", "16"], "geometry.prob_hi": ["1", "1", "1"],
            "nyx.do_hydro": ["0"], "nyx.particle_init_type": ["AsciiFile"],
            "nyx.ascii_particle_file": ["p.ascii"]}
    cfg = run_config(dict(base), str(tmp_path))
    assert cfg.n == 16 and cfg.L == 1.0 and cfg.particle_format == "ascii"
    for key, val, msg in (("nyx.do_hydro", ["1"], "do_hydro"), ("amr.max_level", ["1"], "max_level"),
                          ("amr.n_cell", ["16", "16", "32"], "cubic"),
                          ("geometry.is_periodic", ["1", "1", "0"], "periodic"),
                          ("nyx.particle_init_type", ["Random"], "not supported"),
                          ("nyx.particle_init_type", ["Cosmological"], "ic-source")):
        d = dict(base)
        d[key] = val
        with pytest.raises(ValueError, match=msg):
            run_config(d, str(tmp_path))


def test_cosmological_init_type(tmp_path):
    """particle_init_type = Cosmological reads cosmo.initDirName, cosmo.ic-source,
    nyx.initial_z and nyx.n_particles, as Nyx::initcosmo does."""
    base = {"amr.n_cell": ["16", "16", "16"], "geometry.prob_hi": ["1", "1", "1"],
            "nyx.do_hydro": ["0"], "nyx.particle_init_type": ["Cosmological"],
            "cosmo.initDirName": ["ics"], "cosmo.ic-source": ["MUSIC"], "nyx.initial_z": ["99"]}
    cfg = run_config(dict(base), str(tmp_path))
    assert cfg.particle_format == "cosmological" and cfg.ic_source == "MUSIC"
    assert cfg.particle_file == os.path.join(str(tmp_path), "ics") and cfg.n_particles == 16
    d = dict(base, **{"cosmo.ic-source": ["nyx"], "nyx.n_particles": ["8", "8", "8"]})
    assert run_config(d, str(tmp_path)).n_particles == 8
    for key, val, msg in (("cosmo.ic-source", ["nyx"], "n_particles"),
                          ("cosmo.initDirName", [], "initDirName"),
                          ("nyx.initial_z", None, "initial_z")):
        d = dict(base)
        if val is None:
            del d[key]
        else:
            d[key] = val
        with pytest.raises(ValueError, match=msg):
            run_config(d, str(tmp_path))


@pytest.mark.skipif(NOHYDRO is None, reason="NYX_REFERENCE (the Nyx source tree) not set")
def test_the_references_dm_only_inputs():
    cfg = run_config(read_inputs(NOHYDRO), os.path.dirname(NOHYDRO))
    assert (cfg.n, cfg.L) == (32, 8.0)
    assert (cfg.OmM, cfg.h, cfg.initial_z) == (0.27, 0.71, 100.0)
    assert cfg.final_a == 1.0 / 3.0                      # nyx.final_z = 2
    assert cfg.particle_format == "binary" and cfg.particle_file.endswith("32.nyx")
    assert os.path.exists(cfg.particle_file)
    assert (cfg.rel_tol, cfg.cfl, cfg.change_max, cfg.relative_max_change_a) == (1e-12, 0.5, 1.1, 0.01)
    with pytest.raises(ValueError, match="do_hydro"):
        run_config(read_inputs(os.path.join(os.path.dirname(NOHYDRO), "inputs")),
                   os.path.dirname(NOHYDRO))


def test_restart_init_type(tmp_path):
    """particle_init_type = Restart takes the DM directory of the plotfile or
    checkpoint that nyx.restart_particle_file names (NyxParticles.cpp:584-586)."""
    base = {"amr.n_cell": ["16", "16", "16"], "geometry.prob_hi": ["1", "1", "1"],
            "nyx.do_hydro": ["0"], "nyx.particle_init_type": ["Restart"],
            "nyx.restart_particle_file": ["plt00100"], "particles.dm_particle_output_ascii": ["1"]}
    cfg = run_config(dict(base), str(tmp_path))
    assert cfg.particle_format == "restart" and cfg.ascii_output
    assert cfg.particle_file == os.path.join(str(tmp_path), "plt00100", "DM")
    d = dict(base)
    del d["nyx.restart_particle_file"]
    with pytest.raises(ValueError, match="restart_particle_file"):
        run_config(d, str(tmp_path))
