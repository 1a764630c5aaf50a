"""The allocation-free deposit (nyxpm_deposit_noalloc) against the allocating
one (nyxpm_deposit), through the C ABI.

nyxpm_deposit_noalloc serves callers that cannot allocate device memory (a host
code whose arena owns the GPU's memory): the caller passes device input and
output buffers, and the sort scratch is a static device array.  Its density must
equal the allocating deposit's bit for bit (tolerance: exact), on calls in a row
-- each call reuses the scratch the one before left behind -- including keys
with far more particles than a warp (summed in lane-strided order).

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
    # two Zel'dovich particle sets, then one with keys far longer than a warp
    rng = np.random.default_rng(11)
    crowd = np.concatenate([0.40 + 0.02 * rng.random((3000, 3)), 0.7 + 0.01 * rng.random((700, 3)),
                            rng.random((20000, 3))])
    cases = [(64, zeldovich_ics(64, 1.0, -2.0, 3, 0.05, rms_disp_cells=0.4).pos, 2e9),
             (48, zeldovich_ics(48, 1.0, -2.5, 4, 0.05, rms_disp_cells=0.4).pos, 3e9),
             (32, crowd, 5e8)]
    for call, (n, pos, mass) in enumerate(cases):
        box = Box(ctx, n, 1.0, len(pos))
        box.upload(pos, np.zeros_like(pos), mass)
        expect = box.deposit()
        box.close()
        x, y, z, rho = _device_arrays(torch, pos, n)
        st = lib.nyxpm_deposit_noalloc(C.c_void_p(x.data_ptr()), C.c_void_p(y.data_ptr()),
                                       C.c_void_p(z.data_ptr()), len(pos), mass, n, 1.0,
                                       C.c_void_p(rho.data_ptr()), C.c_void_p(stream), err, len(err))
        assert st == 0, err.value.decode()
        torch.cuda.synchronize()
        got = rho.cpu().numpy()
        assert np.array_equal(got, expect), (call, float(np.nanmax(np.abs(got - expect))))
    # sizes beyond the static scratch are refused with a message, nothing launched
    st = lib.nyxpm_deposit_noalloc(C.c_void_p(x.data_ptr()), C.c_void_p(y.data_ptr()),
                                   C.c_void_p(z.data_ptr()), len(pos), mass, 128, 1.0,
                                   C.c_void_p(rho.data_ptr()), C.c_void_p(stream), err, len(err))
    assert st == 1 and b"64" in err.value
    ctx.close()


@pytest.mark.skipif(not gpu_available(), reason="no GPU")
def test_noalloc_deposit_other_length_own_stream_no_device_memory_taken():
    """A box of side 7.5 (dx and the density scale not powers of two) on a stream
    the caller created: equal to the allocating deposit bit for bit on two calls
    in a row, and the calls after the first take no device memory (free bytes
    unchanged).  A non-finite position is refused, as nyxpm_deposit refuses it."""
    import torch
    from nyx_gb300 import _lib
    from nyx_gb300.ics import zeldovich_ics
    from nyx_gb300.pm import Box, Context

    lib = _lib.load()
    ctx = Context(device=0)
    err = C.create_string_buffer(256)
    L, n, mass = 7.5, 40, 1.7e10
    pos = zeldovich_ics(n, L, -2.0, 21, 0.05, rms_disp_cells=0.5).pos
    box = Box(ctx, n, L, len(pos))
    box.upload(pos, np.zeros_like(pos), mass)
    expect = box.deposit()
    box.close()
    x, y, z, rho = _device_arrays(torch, pos, n)
    side = torch.cuda.Stream(device=0)
    torch.cuda.synchronize()

    def call(xp=x):
        return lib.nyxpm_deposit_noalloc(C.c_void_p(xp.data_ptr()), C.c_void_p(y.data_ptr()),
                                         C.c_void_p(z.data_ptr()), len(pos), mass, n, L,
                                         C.c_void_p(rho.data_ptr()), C.c_void_p(side.cuda_stream),
                                         err, len(err))

    assert call() == 0, err.value.decode()        # the first call sets up the device
    torch.cuda.synchronize()
    free0 = torch.cuda.mem_get_info(0)[0]
    for _ in range(2):
        rho.fill_(float("nan"))
        torch.cuda.synchronize()
        assert call() == 0, err.value.decode()
        side.synchronize()
        assert np.array_equal(rho.cpu().numpy(), expect)
    torch.cuda.synchronize()
    assert torch.cuda.mem_get_info(0)[0] == free0
    bad = x.clone()
    bad[len(pos) // 2] = float("nan")
    torch.cuda.synchronize()
    assert call(bad) == 1 and b"non-finite" in err.value
    ctx.close()


@pytest.mark.skipif(not gpu_available(), reason="no GPU")
def test_noalloc_deposit_captured_in_a_cuda_graph():
    """After one call on the device, the call can be captured into a CUDA graph
    (it then only enqueues: no read-back, no wait) and every replay writes the
    allocating deposit's density, bit for bit."""
    import torch
    from nyx_gb300 import _lib
    from nyx_gb300.ics import zeldovich_ics
    from nyx_gb300.pm import Box, Context

    lib = _lib.load()
    ctx = Context(device=0)
    err = C.create_string_buffer(256)
    L, n, mass = 2.0, 32, 4e9
    pos = zeldovich_ics(n, L, -2.0, 8, 0.05, rms_disp_cells=0.5).pos
    box = Box(ctx, n, L, len(pos))
    box.upload(pos, np.zeros_like(pos), mass)
    expect = box.deposit()
    box.close()
    x, y, z, rho = _device_arrays(torch, pos, n)

    def call(stream):
        return lib.nyxpm_deposit_noalloc(C.c_void_p(x.data_ptr()), C.c_void_p(y.data_ptr()),
                                         C.c_void_p(z.data_ptr()), len(pos), mass, n, L,
                                         C.c_void_p(rho.data_ptr()), C.c_void_p(stream), err, len(err))

    assert call(torch.cuda.current_stream(0).cuda_stream) == 0, err.value.decode()
    torch.cuda.synchronize()
    graph = torch.cuda.CUDAGraph()
    side = torch.cuda.Stream(device=0)
    with torch.cuda.graph(graph, stream=side, capture_error_mode="thread_local"):
        st = call(torch.cuda.current_stream(0).cuda_stream)
    assert st == 0, err.value.decode()
    for _ in range(2):
        rho.fill_(float("nan"))
        graph.replay()
        torch.cuda.synchronize()
        assert np.array_equal(rho.cpu().numpy(), expect)
    del graph
    ctx.close()
