"""The allocation-free deposit (nyxpm_deposit_noalloc) against the allocating
one (nyxpm_deposit), through the C ABI.

nyxpm_deposit_noalloc serves callers that cannot allocate device memory (a host
code whose arena owns the GPU's memory): the caller passes device input and
output buffers, and the sort scratch is a static device array.  Its density must
equal the allocating deposit's bit for bit (tolerance: exact), on two calls in a
row -- the second call reuses the scratch the first one left behind.

This file is collected last so that a failure here comes after every other test.
"""
from __future__ import annotations

import ctypes as C

import numpy as np
import pytest

from tests.conftest import gpu_available

pytestmark = pytest.mark.gpu


def _device_arrays(torch, pos, n):
    dev = torch.device("cuda", 0)
    x = torch.tensor(np.ascontiguousarray(pos[:, 0]), dtype=torch.float64, device=dev)
    y = torch.tensor(np.ascontiguousarray(pos[:, 1]), dtype=torch.float64, device=dev)
    z = torch.tensor(np.ascontiguousarray(pos[:, 2]), dtype=torch.float64, device=dev)
    rho = torch.full((n ** 3,), float("nan"), dtype=torch.float64, device=dev)
    return x, y, z, rho


@pytest.mark.skipif(not gpu_available(), reason="no GPU")
def test_noalloc_deposit_equals_allocating_deposit_twice():
    import torch
    from nyx_gb300 import _lib
    from nyx_gb300.ics import zeldovich_ics
    from nyx_gb300.pm import Box, Context

    lib = _lib.load()
    ctx = Context(device=0)
    err = C.create_string_buffer(256)
    stream = torch.cuda.current_stream(0).cuda_stream
    for call, (n, seed, slope) in enumerate([(64, 3, -2.0), (48, 4, -2.5)]):
        ic = zeldovich_ics(n, 1.0, slope, seed, 0.05, rms_disp_cells=0.4)
        box = Box(ctx, n, 1.0, len(ic.pos))
        box.upload(ic.pos, ic.vel, ic.mass)
        expect = box.deposit()
        box.close()
        x, y, z, rho = _device_arrays(torch, ic.pos, n)
        st = lib.nyxpm_deposit_noalloc(C.c_void_p(x.data_ptr()), C.c_void_p(y.data_ptr()),
                                       C.c_void_p(z.data_ptr()), len(ic.pos), ic.mass, n, 1.0,
                                       C.c_void_p(rho.data_ptr()), C.c_void_p(stream), err, len(err))
        assert st == 0, err.value.decode()
        torch.cuda.synchronize()
        got = rho.cpu().numpy()
        assert np.array_equal(got, expect), (call, float(np.nanmax(np.abs(got - expect))))
    # sizes beyond the static scratch are refused with a message, nothing launched
    st = lib.nyxpm_deposit_noalloc(C.c_void_p(x.data_ptr()), C.c_void_p(y.data_ptr()),
                                   C.c_void_p(z.data_ptr()), len(ic.pos), ic.mass, 128, 1.0,
                                   C.c_void_p(rho.data_ptr()), C.c_void_p(stream), err, len(err))
    assert st == 1 and b"64" in err.value
    ctx.close()
