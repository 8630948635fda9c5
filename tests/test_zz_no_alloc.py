"""gb_go_inventory_noalloc (static device scratch, no allocation) returns what
gb_go_inventory returns, bit for bit, on two calls in a row, before and after steps, for
the FP64 and the FP32-flux forms, and the device's free memory is the same before and
after its calls; a handle over its tracer limit gets GB_GO_ERANGE.

It is the entry point for host models that cannot allocate device memory inside their time
loop (memory reserved up front by a pool they do not own, or other streams that a
device-synchronising cudaMalloc/cudaFree would stall)."""
import ctypes as C
import ctypes.util
import os

import numpy as np
import pytest

from cgenie_gb300 import abi, grid

pytestmark = pytest.mark.gpu


def _cudart():
    """The CUDA runtime as a shared library (the product links its own statically; both
    use the device's primary context)."""
    names = [os.path.join(os.environ.get("CUDA_HOME", "/usr/local/cuda"), "lib64", "libcudart.so"),
             "libcudart.so.13", ctypes.util.find_library("cudart")]
    for n in names:
        if not n:
            continue
        try:
            return C.CDLL(n)
        except OSError:
            continue
    pytest.fail("libcudart not found for cudaMemGetInfo")


def _free_bytes(rt, device):
    assert rt.cudaSetDevice(device) == 0
    free, total = C.c_size_t(0), C.c_size_t(0)
    assert rt.cudaMemGetInfo(C.byref(free), C.byref(total)) == 0
    return free.value


def _pair(g, lib):
    L = g.m.maxl
    a = np.zeros(L)
    b = np.zeros(L)
    dp = C.POINTER(C.c_double)
    assert lib.gb_go_inventory(g.h, a.ctypes.data_as(dp)) == 0
    assert lib.gb_go_inventory_noalloc(g.h, b.ctypes.data_as(dp)) == 0
    return a, b


@pytest.mark.parametrize("precision", [abi.GB_GO_FP64, abi.GB_GO_FP32FLUX], ids=["fp64", "fp32flux"])
def test_noalloc_inventory_equals_inventory(gpu_lib, precision):
    from cgenie_gb300.goldstein import new_member_run
    m = grid.make_member(grid.MemberConfig(maxi=36, maxj=36, maxk=16, maxl=9, seed=81, tracer_kind="bgc"))
    g = new_member_run(m, precision=precision)
    rt = _cudart()
    dp = C.POINTER(C.c_double)
    for steps in (0, 7):
        g.tstepo(steps)
        for _ in range(2):   # two calls in a row
            a, b = _pair(g, g.lib)
            assert np.array_equal(a, b), (a, b)
            assert np.all(np.isfinite(b)) and np.any(b != 0.0)
        # no device memory taken by the entry point itself (its kernels are loaded by now)
        g.sync()
        free0 = _free_bytes(rt, 0)
        c = np.zeros(m.maxl)
        for _ in range(2):
            assert g.lib.gb_go_inventory_noalloc(g.h, c.ctypes.data_as(dp)) == 0
        free1 = _free_bytes(rt, 0)
        assert free1 == free0, (free0, free1)
        assert np.array_equal(c, b)
    g.close()


def test_noalloc_rejects_more_than_64_tracers(gpu_lib):
    from cgenie_gb300.goldstein import new_member_run
    m = grid.make_member(grid.MemberConfig(maxi=8, maxj=6, maxk=4, maxl=65, seed=82, tracer_kind="bgc"))
    g = new_member_run(m, precision=abi.GB_GO_FP64)
    out = np.zeros(m.maxl)
    rc = g.lib.gb_go_inventory_noalloc(g.h, out.ctypes.data_as(C.POINTER(C.c_double)))
    assert rc == abi.GB_GO_ERANGE
    assert b"64 tracers" in g.lib.gb_go_last_error(g.h)
    # the allocating entry point still takes it
    assert np.all(np.isfinite(g.inventory()))
    g.close()
