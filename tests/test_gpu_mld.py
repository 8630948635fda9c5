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


def test_mixed_layer_in_ensembles_within_fp32_bars(gpu_lib):
    """imld = 1 members in the batched split-precision form, in a batch with imld = 0 members:
    the column pass runs co and then the mixed layer in FP64 on the FP64 state, with the
    previous step's rho(maxk) kept per column.  Against each member's FP64 run (bit-exact to
    the oracle above): T and S within 1e-11, every tracer within 1e-6 (per tracer, relative to
    its largest magnitude), convection counts and mixed-layer levels equal, depths within 1e-9;
    also after a change of the wind mixing energy.  The imld = 0 batch-mates equal their runs
    in a batch of their own, bit for bit."""
    from cgenie_gb300.ensemble import Ensemble
    from cgenie_gb300.goldstein import new_member_run
    from test_gpu_long import per_tracer_errors
    mld_mems = [grid.make_member(grid.MemberConfig(**c)) for c in CASES.values()]
    plain = [grid.make_member(c) for c in grid.ensemble_configs(n=4, seed=31)]
    ens = Ensemble(use_graph=True)
    ids = ens.add_many(mld_mems + plain)
    alone = Ensemble(use_graph=True)
    ids_alone = alone.add_many(plain)
    runs = [new_member_run(m, precision=abi.GB_GO_FP64) for m in mld_mems]
    rng = np.random.default_rng(11)
    winds = [np.ascontiguousarray(m.mldketau * rng.uniform(0.0, 3.0, m.mldketau.shape)) for m in mld_mems]
    for phase in range(2):
        ens.step(15)
        alone.step(15)
        for n, (m, g) in enumerate(zip(mld_mems, runs)):
            g.tstepo(15)
            out = ens.download(ids[n])
            ref = g.download()
            err = per_tracer_errors(m, out["ts"], ref["ts"])
            assert np.all(err[:2] <= 1e-11), (n, phase, err)
            assert np.all(err <= 1e-6), (n, phase, err)
            assert np.array_equal(out["cost"], ref["cost"]), (n, phase)
            mld, mldk = ens.download_mld(ids[n])
            rmld, rmldk = g.download_mld()
            assert np.array_equal(mldk, rmldk), (n, phase)
            assert np.max(np.abs(mld - rmld)) <= 1e-9 * max(np.max(np.abs(rmld)), 1e-30), (n, phase)
            assert ens.status(ids[n]) == 0
            if phase == 0:
                ens.set_mld_wind(ids[n], winds[n])
                g.set_mld_wind(winds[n])
        for mid, mida in zip(ids[len(mld_mems):], ids_alone):
            a, b = ens.download(mid), alone.download(mida)
            assert np.array_equal(a["ts"], b["ts"]) and np.array_equal(a["cost"], b["cost"])
    wet = mld_mems[0].k1[1:-1, 1:-1] <= mld_mems[0].maxk
    assert np.any(ens.download_mld(ids[0])[1][wet] < mld_mems[0].maxk - 1)
    with pytest.raises(Exception):
        ens.download_mld(ids[len(mld_mems)])
    for g in runs:
        g.close()
    ens.close()
    alone.close()


@pytest.mark.parametrize("name", list(CASES))
def test_mixed_layer_split_precision_handle(gpu_lib, name):
    """imld = 1 on a single grid in the split-precision form, against the same grid in the FP64
    form (bit-exact to the oracle above), including a first step whose uploaded ts differs from
    ts1 at the surface and a change of the wind energy: T and S within 1e-11, every tracer
    within 1e-6, convection counts and mixed-layer levels equal, depths within 1e-9."""
    from cgenie_gb300.goldstein import new_member_run
    from test_gpu_long import per_tracer_errors
    m = grid.make_member(grid.MemberConfig(**CASES[name]))
    kk = np.arange(m.maxk + 2)[:, None, None]
    wet_top = (kk == m.maxk) & (m.k1[None] <= m.maxk)
    m.ts[..., 0] = np.where(wet_top, m.ts[..., 0] + 0.25, m.ts[..., 0])
    f = new_member_run(m, precision=abi.GB_GO_FP32FLUX)
    g = new_member_run(m, precision=abi.GB_GO_FP64)
    rng = np.random.default_rng(13)
    wind = np.ascontiguousarray(m.mldketau * rng.uniform(0.0, 3.0, m.mldketau.shape))
    for phase in range(2):
        f.tstepo(9)
        g.tstepo(9)
        a, b = f.download(), g.download()
        err = per_tracer_errors(m, a["ts"], b["ts"])
        assert np.all(err[:2] <= 1e-11), (phase, err)
        assert np.all(err <= 1e-6), (phase, err)
        assert np.array_equal(a["cost"], b["cost"]), phase
        mld, mldk = f.download_mld()
        rmld, rmldk = g.download_mld()
        assert np.array_equal(mldk, rmldk), phase
        assert np.max(np.abs(mld - rmld)) <= 1e-9 * max(np.max(np.abs(rmld)), 1e-30), phase
        f.set_mld_wind(wind)
        g.set_mld_wind(wind)
    f.close()
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
