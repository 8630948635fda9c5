"""Config 5 at full size (360x180x32, 24 tracers): the FP64 form equals the oracle bit for
bit over 3 steps; the FP32-flux form stays within the per-tracer bar of the FP64 form
(itself equal to the oracle) over the configuration's 500 steps and conserves the
inventory."""
import numpy as np
import pytest

from cgenie_gb300 import abi, grid

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def c5():
    return grid.make_member(grid.config_c5())


def _wet(m):
    kk = np.arange(m.maxk + 2)[:, None, None]
    w = (kk >= m.k1[None]) & (kk >= 1) & (kk <= m.maxk)
    w[:, 0, :] = w[:, -1, :] = False
    w[:, :, 0] = w[:, :, -1] = False
    return w


def test_c5_fp64_equals_oracle(gpu_lib, oracle, c5):
    from cgenie_gb300.goldstein import new_member_run
    ref = oracle.OracleState(c5)
    ref.step(3)
    g = new_member_run(c5, precision=abi.GB_GO_FP64)
    g.tstepo(3)
    out = g.download()
    g.close()
    assert np.array_equal(out["ts"], ref.ts)
    assert np.array_equal(out["rho"], ref.rho)
    assert np.array_equal(out["cost"], ref.cost)


def test_c5_fp32flux_within_bar_and_conservative(gpu_lib, c5):
    from cgenie_gb300.goldstein import new_member_run
    steps = 500
    g64 = new_member_run(c5, precision=abi.GB_GO_FP64)
    g64.tstepo(steps)
    ref = g64.download()
    g64.close()
    g = new_member_run(c5, precision=abi.GB_GO_FP32FLUX)
    inv0 = g.inventory()
    g.tstepo(steps)
    out = g.download()
    inv1 = g.inventory()
    g.close()
    w = _wet(c5)
    for l in range(c5.maxl):
        a, b = out["ts"][..., l][w], ref["ts"][..., l][w]
        err = np.max(np.abs(a - b)) / np.max(np.abs(b))
        assert err <= (1e-9 if l < 2 else 1e-6), (l, err)
    assert np.all(np.abs(inv1 - inv0) <= 1e-12 * np.abs(inv0))
