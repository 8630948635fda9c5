"""The configurations at the lengths they are stated for.

* The batched ensemble (256 seeded members, FP32 transfers and FP64 state) is checked after
  1000 steps, per tracer, against each member's FP64 run: nine members of the workload (per
  grid shape the fewest, the most and a middle tracer count, so 2 and 24 tracers), stepped
  together in one batch.  The FP64 form is the reference arithmetic bit for bit (checked
  against the oracle here and in test_gpu_fp64.py).
* The isoneutral single member (36x36x16, 17 tracers) in the FP64 form equals the oracle bit
  for bit after its 1000 steps.

Bars, per tracer, error = max|x - x_fp64| / max|x_fp64| over wet cells: T and S <= 1e-11,
every tracer <= 1e-6; convection counts equal; inventory drift <= 1e-12 relative."""
import numpy as np
import pytest

from cgenie_gb300 import abi, grid

pytestmark = pytest.mark.gpu

TOL_TS = 1e-11
TOL_REL = 1e-6
TOL_CONS = 1e-12


def per_tracer_errors(m, ts, ref):
    kk = np.arange(m.maxk + 2)[:, None, None]
    w = (kk >= m.k1[None]) & (kk >= 1) & (kk <= m.maxk)
    w[:, 0, :] = w[:, -1, :] = False
    w[:, :, 0] = w[:, :, -1] = False
    return np.array([float(np.max(np.abs(ts[..., l][w] - ref[..., l][w])) / max(np.max(np.abs(ref[..., l][w])), 1e-300))
                     for l in range(m.maxl)])


def test_ensemble256_sample_1000_steps_per_tracer(gpu_lib):
    from cgenie_gb300.ensemble import Ensemble
    from cgenie_gb300.goldstein import new_member_run
    cfgs = grid.ensemble_configs(256, seed=3)
    pick = grid.error_sample(cfgs)
    assert {cfgs[n].maxl for n in pick} >= {2, 24}
    mems = [grid.make_member(cfgs[n]) for n in pick]
    ens = Ensemble(use_graph=True)
    ids = [ens.add(m) for m in mems]
    inv0 = [ens.inventory(i) for i in ids]
    for _ in range(4):
        ens.step(250)
    worst = np.zeros(24)
    for m, i, v0 in zip(mems, ids, inv0):
        out = ens.download(i)
        g = new_member_run(m, precision=abi.GB_GO_FP64)
        g.tstepo(1000)
        ref = g.download()
        g.close()
        err = per_tracer_errors(m, out["ts"], ref["ts"])
        worst[:m.maxl] = np.maximum(worst[:m.maxl], err)
        assert np.all(err[:2] <= TOL_TS), (m.maxi, m.maxj, m.maxk, m.maxl, err[:2])
        assert np.all(err <= TOL_REL), (m.maxi, m.maxj, m.maxk, m.maxl, err)
        assert np.array_equal(out["cost"], ref["cost"]), "convection counts differ"
        v1 = ens.inventory(i)
        assert np.all(np.abs(v1 - v0) <= TOL_CONS * np.abs(v0)), (v0, v1)
        assert ens.status(i) == 0
    ens.close()
    print("ensemble256 sample, 1000 steps, per-tracer max error:", " ".join(f"{e:.1e}" for e in worst))


def test_config2_fp64_1000_steps_equals_oracle(gpu_lib, oracle):
    from cgenie_gb300.goldstein import new_member_run
    m = grid.make_member(grid.config_c2())
    ref = oracle.OracleState(m)
    ref.step(1000)
    g = new_member_run(m, precision=abi.GB_GO_FP64)
    for n in (1, 499, 500):
        g.tstepo(n)
    out = g.download()
    g.close()
    for name in ("ts", "ts1", "rho", "cost", "icosd"):
        assert np.array_equal(out[name], getattr(ref, name)), name
    assert out["dmax"] == ref.dmax.value and out["limps"] == ref.limps.value
