"""The reference's own bathymetries (tests/golden/masks: worbe2, 36x36 with 8 levels; worjh2,
36x36 with 16 levels; one island each, with its path), read as initialise_goldstein reads
them (src/goldstein/goldstein.f90:1107-1123, 1502-1573), under seeded tracers and
divergence-free velocities:

* CPU: the readers (periodic halo, land codes, landmass labels, path points on wet cells),
  and the oracle's conservation on these grids;
* GPU: the FP64 form equals the oracle bit for bit; the FP32-flux form and a batch of both
  masks stay within the split-precision bars; the momentum step with the real island path
  matches the momentum oracle within 1e-9."""
import os

import numpy as np
import pytest

from cgenie_gb300 import abi, grid

HERE = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden", "masks")
MASKS = {"worbe2": 8, "worjh2": 16}


def cfg(name, maxl=5, seed=7, **kw):
    return grid.MemberConfig(maxi=36, maxj=36, maxk=MASKS[name], maxl=maxl, seed=seed, mask="file",
                             mask_file=os.path.join(HERE, name), tracer_kind="bgc", **kw)


def wet(m):
    kk = np.arange(m.maxk + 2)[:, None, None]
    w = (kk >= m.k1[None]) & (kk >= 1) & (kk <= m.maxk)
    w[:, 0, :] = w[:, -1, :] = False
    w[:, :, 0] = w[:, :, -1] = False
    return w


@pytest.mark.parametrize("name", sorted(MASKS))
def test_readers(name):
    maxk = MASKS[name]
    k1 = grid.read_k1(os.path.join(HERE, name + ".k1"), 36, 36)
    assert k1.shape == (38, 38)
    assert np.array_equal(k1[:, 0], k1[:, 36]) and np.array_equal(k1[:, 37], k1[:, 1])
    assert np.all(k1[0] > maxk) and np.all(k1[37] > maxk)          # the boundary rows are land
    assert np.any(k1 >= 90) and 0.2 < np.mean(k1[1:37, 1:37] > maxk) < 0.5
    ps = grid.read_psiles(os.path.join(HERE, name + ".psiles"), 36, 36)
    isles = int(ps.max()) - 1
    assert isles == 1
    npi, paths = grid.read_paths(os.path.join(HERE, name + ".paths"), isles)
    assert list(npi) == [len(p) for p in paths] == [36]
    for (l_, i_, j_) in paths[0]:
        assert abs(l_) in (1, 2) and k1[j_, i_] <= maxk
    # a psi point is labelled land (> 0) only where one of its four cells is land
    for j in range(37):
        for i in range(1, 37):
            dry = max(k1[j, i], k1[j, i + 1], k1[j + 1, i], k1[j + 1, i + 1]) > maxk
            if ps[(i - 1) + j * 36] > 0:
                assert dry


@pytest.mark.parametrize("name", sorted(MASKS))
def test_oracle_conserves_on_real_mask(oracle, name):
    m = grid.make_member(cfg(name, diso=True, slope_max=1e-3))
    s = oracle.OracleState(m)
    inv0 = s.inventory()
    s.step(20)
    assert np.all(np.abs(s.inventory() - inv0) <= 1e-12 * np.abs(inv0))


@pytest.mark.gpu
@pytest.mark.parametrize("name", sorted(MASKS))
def test_fp64_equals_oracle_on_real_mask(gpu_lib, oracle, name):
    from cgenie_gb300.goldstein import new_member_run
    m = grid.make_member(cfg(name, maxl=6, diso=True, slope_max=1e-3))
    ref = oracle.OracleState(m)
    ref.step(100)
    g = new_member_run(m, precision=abi.GB_GO_FP64)
    g.tstepo(100)
    out = g.download()
    g.close()
    for n in ("ts", "ts1", "rho", "cost", "icosd"):
        assert np.array_equal(out[n], getattr(ref, n)), n
    assert out["dmax"] == ref.dmax.value and out["limps"] == ref.limps.value


@pytest.mark.gpu
def test_fp32flux_batch_on_real_masks(gpu_lib, oracle):
    from cgenie_gb300.ensemble import Ensemble
    mems = [grid.make_member(cfg("worbe2", maxl=24, seed=8)), grid.make_member(cfg("worjh2", maxl=13, seed=9))]
    ens = Ensemble(use_graph=True)
    ids = [ens.add(m) for m in mems]
    inv0 = [ens.inventory(i) for i in ids]
    ens.step(200)
    for m, i, v0 in zip(mems, ids, inv0):
        ref = oracle.OracleState(m)
        ref.step(200)
        out = ens.download(i)
        w = wet(m)
        for l in range(m.maxl):
            a, b = out["ts"][..., l][w], ref.ts[..., l][w]
            err = np.max(np.abs(a - b)) / np.max(np.abs(b))
            assert err <= (1e-11 if l < 2 else 1e-6), (m.maxk, l, err)
        assert np.array_equal(out["cost"], ref.cost)
        v1 = ens.inventory(i)
        assert np.all(np.abs(v1 - v0) <= 1e-12 * np.abs(v0))
        assert ens.status(i) == 0
    ens.close()


@pytest.mark.gpu
@pytest.mark.parametrize("name", sorted(MASKS))
def test_momentum_on_real_mask(gpu_lib, name):
    from cgenie_gb300 import momentum
    from cgenie_gb300.goldstein import new_member_run
    from oracle import oracle_lib as ol
    m = grid.make_member(cfg(name, maxl=2))
    c = momentum.make_case(m, seed=5)
    assert c.isles == 1
    g = new_member_run(m)
    mo = momentum.Momentum(c)
    mo.set_wind()
    o = ol.OracleMomentum(c)
    for _ in range(3):
        mo.step(g)
        o.step(m.rho)
    out, ref = mo.download(), o.state()
    for n in ("psi", "ub", "u", "u1"):
        err = np.abs(out[n] - ref[n]).max() / max(np.abs(ref[n]).max(), 1e-300)
        assert err <= 1e-9, (n, err)
    mo.close()
    g.close()
