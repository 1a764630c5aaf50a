"""CPU checks of the C ABI: the library builds, loads and exports every symbol
include/nyxpm.h declares; host-only entry points (a(t), sizes) agree with the
oracle.  No kernel is launched."""
from __future__ import annotations

import ctypes as C
import os
import re

import pytest

from nyx_gb300 import _lib as L
from oracle import oracle as O
from tests.conftest import gpu_available

REPO = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def header_functions():
    txt = open(os.path.join(REPO, "include", "nyxpm.h")).read()
    txt = re.sub(r"/\*.*?\*/", "", txt, flags=re.S)
    return sorted(set(re.findall(r"\b(nyxpm_[a-z_0-9]+)\s*\(", txt)))


def test_header_declares_expected_entry_points():
    names = header_functions()
    assert set(L.EXPORTS) == set(names), set(L.EXPORTS) ^ set(names)


def test_library_loads_and_exports_every_symbol():
    lib = L.load()
    for name in header_functions():
        assert hasattr(lib, name), name
    assert lib.nyxpm_abi_version() == 2


def test_default_params_match_reference_constants():
    lib = L.load()
    p = L.Params()
    lib.nyxpm_default_params(C.byref(p))
    assert p.gconst == O.gconst()
    assert p.rel_tol == 1e-10 and p.nu1 == 2 and p.nu2 == 2 and p.max_vcycles == 100


def test_a_of_t_equals_oracle_exactly():
    lib = L.load()
    p = L.Params()
    lib.nyxpm_default_params(C.byref(p))
    for a0, dt in ((0.02, 1e-5), (0.1, 3e-4), (0.4, 1e-3)):
        assert lib.nyxpm_integrate_a(C.byref(p), a0, dt) == O.integrate_a(1.0, 0.0, 0.675, a0, dt)
        a1 = a0 * 1.05
        assert lib.nyxpm_dt_for_da(C.byref(p), a0, a1, 2 * dt) == O.dt_for_da(1.0, 0.0, 0.675, a0, a1, 2 * dt)


def test_box_bytes_scales():
    lib = L.load()
    small = lib.nyxpm_box_bytes(64, 64 ** 3, L.NYXPM_FP64)
    big = lib.nyxpm_box_bytes(256, 256 ** 3, L.NYXPM_FP64)
    assert 50 < big / small < 70
    assert lib.nyxpm_box_bytes(256, 256 ** 3, L.NYXPM_MIXED) < big


@pytest.mark.skipif(gpu_available(), reason="checks the no-device error path")
def test_create_without_device_reports_no_device():
    lib = L.load()
    p = L.Params()
    lib.nyxpm_default_params(C.byref(p))
    h = C.c_void_p()
    st = lib.nyxpm_create(C.byref(p), C.byref(h))
    assert st == 6 and not h.value


def test_null_handles_are_rejected():
    lib = L.load()
    assert lib.nyxpm_synchronize(None) == 1
    assert lib.nyxpm_deposit(None, None, None) == 1
    assert lib.nyxpm_step(None, None, 0.1, 0.2, 1e-3, 0, None) == 1


def test_dt_params_defaults_are_the_references():
    lib = L.load()
    dp = L.DtParams()
    lib.nyxpm_default_dt_params(C.byref(dp))
    assert (dp.cfl, dp.change_max, dp.relative_max_change_a) == (0.5, 1.1, 0.01)
    assert dp.absolute_max_change_a < 0 and dp.final_a < 0 and dp.stop_time < 0 and dp.dt_binpow < 0


@pytest.mark.parametrize("OmM,OmR,h", [(1.0, 0.0, 0.675), (0.3, 1e-4, 0.7)])
def test_comoving_time_step_limit_equals_oracle_exactly(OmM, OmR, h):
    """Nyx::comoving_est_time_step on the host: the relative and absolute a-change
    limits, final_a and the power-of-two binning, bit for bit against the oracle."""
    lib = L.load()
    p = L.Params()
    lib.nyxpm_default_params(C.byref(p))
    p.comoving_OmM, p.comoving_OmR, p.comoving_h = OmM, OmR, h
    cases = 0
    for a in (0.01, 0.02, 0.1, 0.45, 0.9):
        for estdt in (1e200, 1e-7, 2e-6, 3e-4):
            for rel, absc in ((0.01, -1.0), (0.05, -1.0), (0.01, 0.0096), (0.01, 0.001)):
                for final_a in (-1.0, 0.5):
                    for binpow in (-1.0, 0.0):
                        dp = L.DtParams()
                        lib.nyxpm_default_dt_params(C.byref(dp))
                        dp.relative_max_change_a, dp.absolute_max_change_a = rel, absc
                        dp.final_a, dp.dt_binpow = final_a, binpow
                        out = C.c_double(0)
                        st = lib.nyxpm_comoving_est_dt(C.byref(p), a, estdt, C.byref(dp), C.byref(out))
                        want, ost = O.comoving_est_dt(OmM, OmR, h, a, estdt, rel, absc, final_a, binpow)
                        assert (st != 0) == (ost != 0), (a, estdt, rel, absc, final_a, binpow)
                        if st == 0:
                            assert out.value == want, (a, estdt, rel, absc, final_a, binpow)
                            assert 0 < out.value <= estdt
                            cases += 1
    assert cases > 200
