"""Tracing calls on the GPU (include/gb_trace.h): the profiler's collection window opens and
closes with a device present, and a run inside the caller's nested task ranges (as the
reference's ITT tasks around its module calls) gives the same state bit for bit as the same run
without them.  Whether a profiler sees the ranges is shown by an NVTX-filtered Nsight Compute
capture, not here: without an attached tool every range call is a no-op."""
import numpy as np
import pytest

from cgenie_gb300 import abi, grid

pytestmark = pytest.mark.gpu


def test_trace_ranges_leave_results_unchanged(gpu_lib):
    from cgenie_gb300.goldstein import new_member_run
    L = gpu_lib
    m = grid.make_member(grid.MemberConfig(maxi=18, maxj=14, maxk=16, maxl=4, seed=91, noise=2.0))

    def run(traced):
        g = new_member_run(m, precision=abi.GB_GO_FP32FLUX)
        if traced:
            d = L.gb_tr_domain_create(b"genie")
            step, ocean = L.gb_tr_string_handle_create(b"timestep"), L.gb_tr_string_handle_create(b"goldstein")
            assert L.gb_tr_resume() == abi.GB_GO_OK
            for _ in range(3):
                L.gb_tr_task_begin(d, step)
                L.gb_tr_task_begin(d, ocean)
                g.tstepo(4)
                L.gb_tr_task_end(d)
                L.gb_tr_task_end(d)
            assert L.gb_tr_pause() == abi.GB_GO_OK
        else:
            g.tstepo(12)
        out = g.download()
        g.close()
        return out

    a, b = run(False), run(True)
    for k in ("ts", "rho", "cost"):
        assert np.array_equal(a[k], b[k]), k
