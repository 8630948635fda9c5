"""GPU parity of the Kraus-Turner mixed layer (imld = 1, goldstein.f90:2294-2390 and
3337-3442) in the FP64 form against the oracle, bit-exact: tracers, rho, convection
counts and the diagnostics mld/mldk, including a change of the wind mixing energy
between steps and a first step whose uploaded ts differs from ts1 at the surface (the
surface-layer energy reads ts, the flux reads ts1)."""
import numpy as np
import pytest

from cgenie_gb300 import abi, grid
from test_gpu_fp64 import assert_same

pytestmark = pytest.mark.gpu

CASES = {
    "partial": dict(maxi=24, maxj=18, maxk=12, maxl=3, seed=201, forcing=1.0, imld=1, mldketau_max=3e-3,
                    mldwindkedec=500.0),
    "deep_ieos_coshuffle_diso": dict(maxi=24, maxj=18, maxk=16, maxl=5, seed=202, forcing=1.0, imld=1,
                                     mldketau_max=1e-2, mldwindkedec=2000.0, ieos=1, iconv=1, noise=2.0,
                                     diso=True, slope_max=1e-3),
    "nowind": dict(maxi=20, maxj=12, maxk=8, maxl=2, seed=203, forcing=1.0, imld=1, mldketau_max=0.0),
}


def oracle_state(oracle, m):
    s = oracle.OracleState(m)
    return s


def gpu_outputs(g):
    out = g.download()
    out["mld"], out["mldk"] = g.download_mld()
    return out


def oracle_outputs(s):
    return dict(ts=s.ts, ts1=s.ts1, rho=s.rho, cost=s.cost, icosd=s.icosd, mld=s.mld, mldk=s.mldk)


@pytest.mark.parametrize("name", list(CASES))
def test_mixed_layer_bitexact(gpu_lib, oracle, name):
    from cgenie_gb300.goldstein import new_member_run
    m = grid.make_member(grid.MemberConfig(**CASES[name]))
    # the first step's surface-layer energy reads the uploaded ts, not ts1
    kk = np.arange(m.maxk + 2)[:, None, None]
    wet_top = (kk == m.maxk) & (m.k1[None] <= m.maxk)
    m.ts[..., 0] = np.where(wet_top, m.ts[..., 0] + 0.25, m.ts[..., 0])
    s = oracle_state(oracle, m)
    g = new_member_run(m)
    s.step(7)
    g.tstepo(3)
    g.tstepo(4)
    out = gpu_outputs(g)
    ref = oracle_outputs(s)
    assert_same(out, ref, ("ts", "ts1", "rho", "cost", "icosd", "mld", "mldk"))
    # new wind mixing energy for both
    rng = np.random.default_rng(7)
    wind = np.ascontiguousarray(m.mldketau * rng.uniform(0.0, 3.0, m.mldketau.shape))
    s.refs.arrays["mldketau"][...] = wind
    g.set_mld_wind(wind)
    s.step(6)
    g.tstepo(6)
    out = gpu_outputs(g)
    ref = oracle_outputs(s)
    assert_same(out, ref, ("ts", "ts1", "rho", "cost", "icosd", "mld", "mldk"))
    wet = m.k1[1:-1, 1:-1] <= m.maxk
    assert np.all(out["mldk"][wet] >= 1)
    if name != "nowind":
        # the scheme deepens some mixed layers below the top level
        assert np.any(out["mldk"][wet] < m.maxk - 1)
    g.close()


def test_mixed_layer_rejections(gpu_lib):
    from cgenie_gb300.goldstein import Goldstein, GoldsteinError
    m = grid.make_member(grid.MemberConfig(**CASES["nowind"]))
    g = Goldstein(m, imld=0)
    with pytest.raises(GoldsteinError) as e:
        g.download_mld()
    assert e.value.code == abi.GB_GO_EINVAL
    with pytest.raises(GoldsteinError) as e:
        g.set_mld_wind(m.mldketau)
    assert e.value.code == abi.GB_GO_EINVAL
    g.close()
    with pytest.raises(GoldsteinError) as e:
        Goldstein(m, precision=abi.GB_GO_FP32FLUX)
    assert e.value.code == abi.GB_GO_EUNSUPPORTED
