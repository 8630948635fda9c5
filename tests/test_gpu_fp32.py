"""GPU checks of the FP32-flux / FP64-state form and the batched ensemble.

Bars (per tracer): relative error against the FP64 oracle
    max over wet cells |x - x_oracle| / max over wet cells |x_oracle|  <= 1e-6
after the stated number of steps, and conservation drift of the compensated
inventory sum(ts*ds*dz) <= 1e-12 relative with zero surface forcing."""
import numpy as np
import pytest

from cgenie_gb300 import abi, grid

pytestmark = pytest.mark.gpu

TOL_REL = 1e-6
TOL_CONS = 1e-12


def wet_mask(m):
    kk = np.arange(m.maxk + 2)[:, None, None]
    return (kk >= m.k1[None]) & (kk >= 1) & (kk <= m.maxk) & (np.arange(m.maxj + 2)[None, :, None] >= 1) & \
        (np.arange(m.maxj + 2)[None, :, None] <= m.maxj) & (np.arange(m.maxi + 2)[None, None, :] >= 1) & \
        (np.arange(m.maxi + 2)[None, None, :] <= m.maxi)


def tracer_errors(m, ts, ref):
    w = wet_mask(m)
    out = []
    for l in range(m.maxl):
        a = ts[..., l][w]
        b = ref[..., l][w]
        out.append(float(np.max(np.abs(a - b)) / max(np.max(np.abs(b)), 1e-300)))
    return np.array(out)


def oracle_ts(oracle, m, steps):
    s = oracle.OracleState(m)
    s.step(steps)
    return s


def run_fp32(m, steps):
    from cgenie_gb300.goldstein import new_member_run
    g = new_member_run(m, precision=abi.GB_GO_FP32FLUX)
    inv0 = g.inventory()
    g.tstepo(steps)
    out = g.download()
    out["inv0"] = inv0
    out["inv1"] = g.inventory()
    g.close()
    return out


@pytest.mark.parametrize("cfg,steps", [
    (grid.config_c1(), 100),
    (grid.config_c2(), 200),
    (grid.MemberConfig(maxi=37, maxj=23, maxk=13, maxl=5, seed=51, diso=True), 50),
    (grid.MemberConfig(maxi=18, maxj=18, maxk=32, maxl=24, seed=52, diso=True, tracer_kind="bgc"), 50),
], ids=["c1", "c2", "odd", "deep24"])
def test_fp32_matches_fp64_oracle(gpu_lib, oracle, cfg, steps):
    m = grid.make_member(cfg)
    ref = oracle_ts(oracle, m, steps)
    out = run_fp32(m, steps)
    err = tracer_errors(m, out["ts"], ref.ts)
    assert np.all(err <= TOL_REL), err
    rel = np.abs(out["inv1"] - out["inv0"]) / np.abs(out["inv0"])
    assert np.all(rel <= TOL_CONS), rel
    # convection diagnostics agree with the oracle (same convecting levels)
    assert np.abs(out["cost"] - ref.cost).max() <= 2


def test_fp32_conservation_1000_steps(gpu_lib):
    m = grid.make_member(grid.config_c2())
    out = run_fp32(m, 1000)
    rel = np.abs(out["inv1"] - out["inv0"]) / np.abs(out["inv0"])
    assert np.all(rel <= TOL_CONS), rel


def test_fp32_forcing_and_branches(gpu_lib, oracle):
    for cfg in [grid.MemberConfig(maxi=18, maxj=14, maxk=8, maxl=3, seed=53, forcing=1.0),
                grid.MemberConfig(maxi=18, maxj=14, maxk=8, maxl=3, seed=54, iconv=1, ieos=1, diso=True, noise=2.0)]:
        m = grid.make_member(cfg)
        ref = oracle_ts(oracle, m, 20)
        out = run_fp32(m, 20)
        err = tracer_errors(m, out["ts"], ref.ts)
        assert np.all(err <= TOL_REL), (cfg, err)


def test_ensemble_alone_equals_in_mix(gpu_lib):
    """A member's result is the same (bit for bit) alone and in a mixed batch."""
    from cgenie_gb300.ensemble import Ensemble
    cfgs = grid.ensemble_configs(n=9, seed=9)
    mems = [grid.make_member(c) for c in cfgs]
    alone = Ensemble()
    aid = alone.add(mems[4])
    alone.step(30)
    a = alone.download(aid)
    alone.close()
    mix = Ensemble()
    ids = [mix.add(m) for m in mems]
    mix.step(30)
    b = mix.download(ids[4])
    assert np.array_equal(a["ts"], b["ts"])
    # staggered admission: a member admitted later runs the same 30 steps
    late = mix.add(mems[4], steps=30)
    mix.step(45)
    c = mix.download(late)
    assert np.array_equal(a["ts"], c["ts"])
    assert mix.remaining(late) == 0
    mix.close()


def test_ensemble_matches_oracle_per_member(gpu_lib, oracle):
    from cgenie_gb300.ensemble import Ensemble
    cfgs = grid.ensemble_configs(n=6, seed=11)
    mems = [grid.make_member(c) for c in cfgs]
    ens = Ensemble(use_graph=True)
    ids = [ens.add(m) for m in mems]
    inv0 = [ens.inventory(i) for i in ids]
    ens.step(20)
    ens.step(20)
    for m, i, v0 in zip(mems, ids, inv0):
        ref = oracle_ts(oracle, m, 40)
        out = ens.download(i)
        err = tracer_errors(m, out["ts"], ref.ts)
        assert np.all(err <= TOL_REL), err
        v1 = ens.inventory(i)
        assert np.all(np.abs(v1 - v0) <= TOL_CONS * np.abs(v0))
        assert ens.status(i) == 0
    ens.close()


def test_ensemble_budget_and_removal(gpu_lib):
    from cgenie_gb300.ensemble import Ensemble
    from cgenie_gb300.goldstein import GoldsteinError
    m = grid.make_member(grid.MemberConfig(maxi=18, maxj=18, maxk=16, maxl=4, seed=55))
    nb = Ensemble.member_bytes(m)
    ens = Ensemble(hbm_budget_bytes=int(2.5 * nb))
    a = ens.add(m)
    b = ens.add(m)
    with pytest.raises(GoldsteinError) as ex:
        ens.add(m)
    assert ex.value.code == abi.GB_GO_ENOMEM
    ens.remove(a)
    c = ens.add(m)
    ens.step(3)
    assert ens.count()[0] == 2
    ens.remove(b)
    ens.remove(c)
    ens.close()
