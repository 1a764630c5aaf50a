"""nyxpm_step_host (upload + step + download in one call, the transfers
overlapped with the step on a second stream, FP64 and mixed boxes) gives the
results of the three calls, bit for bit; a non-finite input is reported as an
error."""
from __future__ import annotations

import numpy as np
import pytest

from nyx_gb300.pm import Box, NyxPMError
from tests.pm_cases import config1_ics, equal_da_schedule

pytestmark = pytest.mark.gpu


@pytest.mark.parametrize("precision,reuse,per_particle_mass",
                         [("fp64", False, False), ("fp64", True, False), ("fp64", False, True),
                          ("mixed", False, False), ("mixed", True, False), ("mixed", False, True)])
def test_host_step_equals_upload_step_download(ctx, precision, reuse, per_particle_mass):
    n = 32
    ic = config1_ics(n, seed=7)
    rng = np.random.default_rng(3)
    mass = (ic.mass * (0.5 + rng.random(len(ic.pos)))) if per_particle_mass else ic.mass
    sched = equal_da_schedule(0.02, 0.05, 3)
    b1 = Box(ctx, n, 1.0, len(ic.pos), precision=precision)
    b2 = Box(ctx, n, 1.0, len(ic.pos), precision=precision)
    for b in (b1, b2):
        b.upload(ic.pos, ic.vel, mass)
        if reuse:
            b.init_field(0.02)
    p1, v1 = ic.pos.copy(), ic.vel.copy()
    p2, v2 = ic.pos.copy(), ic.vel.copy()
    for a0, a1, dt in sched:
        b1.upload(p1, v1, mass)
        i1 = b1.step(a0, a1, dt, reuse_field=reuse)
        p1, v1 = b1.download()
        i2 = b2.step_host(p2, v2, mass, a0, a1, dt, reuse_field=reuse)
        assert i1 == i2
        assert np.array_equal(p1, p2) and np.array_equal(v1, v2)
    assert np.array_equal(b1.get_phi(), b2.get_phi())
    b1.close()
    b2.close()


@pytest.mark.parametrize("precision", ["fp64", "mixed"])
def test_host_step_reports_non_finite_input(ctx, precision):
    n = 16
    ic = config1_ics(n, seed=8)
    b = Box(ctx, n, 1.0, len(ic.pos), precision=precision)
    b.upload(ic.pos, ic.vel, ic.mass)
    for which in ("vel", "pos"):
        p, v = ic.pos.copy(), ic.vel.copy()
        (v if which == "vel" else p)[5, 1] = np.nan
        with pytest.raises(NyxPMError) as e:
            b.step_host(p, v, ic.mass, 0.02, 0.021, 1e-3)
        assert "non-finite" in str(e.value)
    b.close()
