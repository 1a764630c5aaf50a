"""The smoke entry point (one FP64 step of a 16^3 box against the oracle) runs
green on the GPU."""
from __future__ import annotations

import pytest

pytestmark = pytest.mark.gpu


def test_smoke_entry_point():
    import __graft_entry__ as g
    g.smoke()
