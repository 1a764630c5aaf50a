"""GPU tests of the continuous-batching server.

* each run's result is bitwise the same served alone and served in a mix of
  concurrent runs that join and leave at different times;
* admission never exceeds the memory budget and every request completes.
"""
from __future__ import annotations

import numpy as np
import pytest

from nyx_gb300.ensemble import Ensemble, box_ics
from nyx_gb300.serving import ContinuousBatchingServer, Request

pytestmark = pytest.mark.gpu


def provider(r: Request):
    return box_ics(r.spec(), 0.02)


def stream():
    sizes = [16, 32, 16, 48, 32, 16, 32, 16]
    steps = [3, 5, 2, 4, 3, 6, 2, 4]
    return [Request(rid=i, arrival=0.0, n=n, nsteps=s, seed=100 + i, slope=-1.5 - 0.1 * i)
            for i, (n, s) in enumerate(zip(sizes, steps))]


def test_served_in_mix_equals_alone(ctx):
    reqs = stream()
    budget = int(sum(Ensemble.box_bytes(r.n, r.np) for r in reqs[:4]) * 1.05)
    srv = ContinuousBatchingServer(ctx, budget, provider, keep_results=True)
    mix = {r.rid: r for r in srv.serve(reqs, realtime=False).results}
    srv.close()
    assert len(mix) == len(reqs)
    for req in reqs:
        one = ContinuousBatchingServer(ctx, Ensemble.box_bytes(req.n, req.np) + (16 << 20), provider,
                                       keep_results=True)
        alone = one.serve([req], realtime=False).results[0]
        one.close()
        got = mix[req.rid]
        assert np.array_equal(got.pos, alone.pos), req
        assert np.array_equal(got.vel, alone.vel), req


def test_admission_by_budget(ctx):
    reqs = [Request(rid=i, arrival=0.0, n=32, nsteps=3, seed=7 + i, slope=-2.0) for i in range(5)]
    one = Ensemble.box_bytes(32, 32 ** 3)
    srv = ContinuousBatchingServer(ctx, int(one * 2.5), provider)
    st = srv.serve(reqs, realtime=False)
    srv.close()
    assert len(st.results) == 5
    assert st.max_active == 2
    assert st.peak_arena_bytes <= one * 2.5
