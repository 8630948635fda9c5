"""gb_go_inventory_noalloc (static device scratch, no allocation) returns what
gb_go_inventory returns, bit for bit, on two calls in a row, before and after steps, for
the FP64 and the FP32-flux forms; a handle over its tracer limit gets GB_GO_ERANGE."""
import ctypes as C

import numpy as np
import pytest

from cgenie_gb300 import abi, grid

pytestmark = pytest.mark.gpu


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
    for steps in (0, 7):
        g.tstepo(steps)
        for _ in range(2):   # two calls in a row
            a, b = _pair(g, g.lib)
            assert np.array_equal(a, b), (a, b)
            assert np.all(np.isfinite(b)) and np.any(b != 0.0)
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
