"""A run started from Nyx particle IC files through the reference-named facade
(DarkMatterParticleContainer.InitFromAsciiFile / InitFromBinaryFile) equals the
oracle started from the same particles."""
from __future__ import annotations

import numpy as np
import pytest

from nyx_gb300.pm import Box, DarkMatterParticleContainer, read_particle_file, write_particle_file
from oracle import oracle as O
from tests.pm_cases import config1_ics, equal_da_schedule, min_image, rel_l2

pytestmark = pytest.mark.gpu


@pytest.mark.parametrize("fmt", ["ascii", "binary"])
def test_run_from_particle_file(ctx, tmp_path, fmt):
    n = 32
    ic = config1_ics(n, seed=5)
    path = tmp_path / f"ics.{fmt}"
    write_particle_file(path, ic.pos, ic.vel, ic.mass, fmt)
    box = Box(ctx, n, 1.0, len(ic.pos))
    dmpc = DarkMatterParticleContainer(box)
    (dmpc.InitFromAsciiFile if fmt == "ascii" else dmpc.InitFromBinaryFile)(path)
    pos, vel, mass = read_particle_file(path, fmt)
    p = O.Particles(pos, vel, mass[0])
    pm = O.PMOracle(n, 1.0, p)
    for a0, a1, dt in equal_da_schedule(0.02, 0.03, 3):
        box.step(a0, a1, dt)
        pm.step(a0, a1, dt)
    gpos, gvel = box.download()
    opos, ovel = p.by_id()
    assert np.linalg.norm(min_image(gpos - opos, 1.0)) / np.linalg.norm(opos) <= 1e-12
    assert rel_l2(gvel, ovel) <= 1e-12
    out = tmp_path / "out.ascii"
    dmpc.WriteAsciiFile(out)
    rp, rv, rm = read_particle_file(out, "ascii")
    assert np.array_equal(rp, gpos) and np.array_equal(rv, gvel)
    box.close()


def test_run_from_cosmological_fields(ctx):
    """Nyx::initcosmo on one level: IC displacement and velocity fields (here the
    Zel'dovich fields of the ICs generator, in box-length units) -> one particle
    per cell on the GPU, then steps equal to the oracle's from the same particles."""
    from nyx_gb300.pm import cosmo_1ppc_particles
    n, L = 32, 1.0
    ic = config1_ics(n, seed=6)
    disp = (ic.pos - ic.lattice + 0.5 * L) % L - 0.5 * L       # displacement of each cell's particle
    vel = ic.vel
    df, vf = [L] * 3, [1.0] * 3
    box = Box(ctx, n, L, n ** 3)
    box.init_cosmo_1ppc(disp.T / L, vel.T, df, vf, ic.mass)
    pos, v = cosmo_1ppc_particles(n, L, disp.T / L, vel.T, df, vf)
    assert np.abs(min_image(pos - ic.pos, L)).max() < 1e-12
    p = O.Particles(pos, v, ic.mass)
    pm = O.PMOracle(n, L, p)
    for a0, a1, dt in equal_da_schedule(0.02, 0.03, 2):
        box.step(a0, a1, dt)
        pm.step(a0, a1, dt)
    gpos, gvel = box.download()
    opos, ovel = p.by_id()
    assert np.linalg.norm(min_image(gpos - opos, L)) / np.linalg.norm(opos) <= 1e-12
    assert rel_l2(gvel, ovel) <= 1e-12
    box.close()
