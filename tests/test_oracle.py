"""CPU checks of the oracle: golden fixtures, agreement of the two restatements,
and known-answer properties of the reference algorithm (goldstein.f90:2280-2842)."""
import glob
import os

import numpy as np
import pytest

import member_io
from cgenie_gb300 import grid
from oracle import goldstein_np as gnp

GOLDEN = sorted(glob.glob(os.path.join(os.path.dirname(__file__), "golden", "*.npz")))


@pytest.mark.parametrize("path", GOLDEN, ids=[os.path.basename(p)[:-4] for p in GOLDEN])
def test_c_oracle_reproduces_golden(oracle, path):
    m, out = member_io.load(path)
    s = oracle.OracleState(m)
    s.step(int(out["steps"]))
    for name in ("ts", "ts1", "rho", "cost", "icosd", "mld", "mldk"):
        if name in out:
            assert np.array_equal(getattr(s, name), out[name]), name
    assert s.dmax.value == float(out["dmax"])
    assert s.limps.value == int(out["limps"])


GOLDEN_NP = GOLDEN[:4] + [p for p in GOLDEN if os.path.basename(p).startswith("mld_")]


@pytest.mark.parametrize("path", GOLDEN_NP, ids=[os.path.basename(p)[:-4] for p in GOLDEN_NP])
def test_numpy_oracle_reproduces_golden(path):
    m, out = member_io.load(path)
    p = gnp.Params(m, m.cfg.diso, m.cfg.ieos, m.cfg.iconv, m.cfg.iediff, m.cfg.imld)
    ts, ts1, rho, cost, icosd = m.copy_state()
    mld = None if m.mld is None else m.mld.copy()
    mldk = None if m.mldk is None else m.mldk.copy()
    dmax, limps = gnp.tstepo(m, p, ts, ts1, rho, m.u, cost, icosd, int(out["steps"]), mld, mldk)
    for name, a in (("ts", ts), ("ts1", ts1), ("rho", rho), ("cost", cost), ("icosd", icosd), ("mld", mld),
                    ("mldk", mldk)):
        if name in out:
            assert np.array_equal(a, out[name]), name
    assert dmax == float(out["dmax"]) and limps == int(out["limps"])


@pytest.mark.parametrize("kw", [
    dict(maxi=36, maxj=36, maxk=16, maxl=2, seed=101),
    dict(maxi=18, maxj=18, maxk=16, maxl=5, seed=102, diso=True, slope_max=1e-3),
    dict(maxi=15, maxj=9, maxk=7, maxl=3, seed=103, iconv=1, ieos=1, diso=True, noise=2.0),
    # Kraus-Turner mixed layer: partial mixing at many depths, mixing to the bottom,
    # too little energy for the first layer (zero wind), thermobaricity and coshuffle
    dict(maxi=18, maxj=14, maxk=12, maxl=3, seed=104, forcing=1.0, imld=1, mldketau_max=3e-3,
         mldwindkedec=500.0),
    dict(maxi=18, maxj=14, maxk=12, maxl=4, seed=105, forcing=1.0, imld=1, mldketau_max=1e-2,
         mldwindkedec=2000.0, ieos=1, iconv=1, noise=2.0, diso=True),
    dict(maxi=15, maxj=9, maxk=7, maxl=2, seed=106, forcing=1.0, imld=1, mldketau_max=0.0),
], ids=["plain", "diso", "coshuffle_ieos", "mld", "mld_ieos_coshuffle_diso", "mld_nowind"])
def test_restatements_agree_bitwise(oracle, kw):
    m = grid.make_member(grid.MemberConfig(**kw))
    s = oracle.OracleState(m)
    s.step(3)
    p = gnp.Params(m, m.cfg.diso, m.cfg.ieos, m.cfg.iconv, m.cfg.iediff, m.cfg.imld)
    ts, ts1, rho, cost, icosd = m.copy_state()
    mld, mldk = m.mld.copy(), m.mldk.copy()
    gnp.tstepo(m, p, ts, ts1, rho, m.u, cost, icosd, 3, mld, mldk)
    assert np.array_equal(s.ts, ts)
    assert np.array_equal(s.ts1, ts1)
    assert np.array_equal(s.rho, rho)
    assert np.array_equal(s.cost, cost)
    assert np.array_equal(s.mld, mld)
    assert np.array_equal(s.mldk, mldk)
    if m.cfg.imld:
        wet = m.k1[1:-1, 1:-1] <= m.maxk
        assert np.all(s.mldk[wet] >= 1)


def test_conservation_zero_forcing(oracle):
    """Flux form telescopes (fw=fe, fs=fn, fb=fa reuse, goldstein.f90:2633-2635) and co
    mixes volume-weighted: with zero surface forcing the inventory sum(ts*ds*dz) is
    conserved to rounding."""
    m = grid.make_member(grid.MemberConfig(maxi=36, maxj=36, maxk=16, maxl=4, seed=7, diso=True,
                                           slope_max=1e-3))
    s = oracle.OracleState(m)
    inv0 = s.inventory()
    s.step(50)
    inv1 = s.inventory()
    rel = np.abs(inv1 - inv0) / np.abs(inv0)
    assert np.all(rel < 1e-12), rel


def test_uniform_field_zero_velocity_invariant(oracle):
    """A uniform stratification-free field with zero velocity and zero forcing is a
    fixed point of the step: every face flux vanishes; equal densities make co mix
    equal values (rho(k(m)) >= rho(k(m-1)) holds with equality), which changes them
    only by the rounding of sum/dzm."""
    m = grid.make_member(grid.MemberConfig(maxi=12, maxj=10, maxk=8, maxl=3, seed=8, umax=0.0, diso=True))
    kk = np.arange(m.maxk + 2)[:, None, None]
    wet = (kk >= m.k1[None]) & (kk >= 1) & (kk <= m.maxk)
    for l, v in enumerate((3.25, 0.5, 7.0)):
        m.ts[..., l] = np.where(wet, v, 0.0)
    m.ts1[...] = m.ts
    s = oracle.OracleState(m)
    s.step(5)
    np.testing.assert_allclose(s.ts[wet], m.ts[wet], rtol=4e-15, atol=0)


def test_co_stable_column_unchanged_and_idempotent(oracle):
    """co conserves the volume-weighted column sums, and a second pass changes the
    state only by rounding: mixed levels hold equal densities, which the
    reference's test rho(k(m)) >= rho(k(m-1)) mixes again (goldstein.f90:2657-2777)."""
    from cgenie_gb300.abi import GridRefs, dptr, iptr
    import ctypes as C
    m = grid.make_member(grid.MemberConfig(maxi=10, maxj=8, maxk=8, maxl=3, seed=9, noise=3.0))
    r = GridRefs(m)
    L = oracle.lib()
    ts = m.ts.copy()
    rho = m.rho.copy()
    cost = np.zeros_like(m.cost)
    icosd = np.zeros_like(m.icosd)
    assert L.gbo_co(C.byref(r.dims), C.byref(r.params), C.byref(r.grid), dptr(ts), dptr(rho), dptr(cost),
                    iptr(icosd)) == 0
    assert cost.sum() > 0  # the noisy state convects
    # volume-weighted column sums conserved
    dz = m.dz
    for j in range(1, m.maxj + 1):
        for i in range(1, m.maxi + 1):
            k1 = m.k1[j, i]
            if k1 > m.maxk:
                continue
            a = (m.ts[k1:m.maxk + 1, j, i, :] * dz[k1 - 1:, None]).sum(0)
            b = (ts[k1:m.maxk + 1, j, i, :] * dz[k1 - 1:, None]).sum(0)
            np.testing.assert_allclose(a, b, rtol=1e-13, atol=1e-15)
    ts2 = ts.copy()
    rho2 = rho.copy()
    cost2 = np.zeros_like(cost)
    assert L.gbo_co(C.byref(r.dims), C.byref(r.params), C.byref(r.grid), dptr(ts2), dptr(rho2), dptr(cost2),
                    iptr(icosd)) == 0
    np.testing.assert_allclose(ts2, ts, rtol=1e-14, atol=1e-300)


def test_eos_matches_formula(oracle):
    import ctypes as C
    ec = grid.eos_coefficients(1)
    ecp = (C.c_double * 5)(*ec)
    L = oracle.lib()
    for t, s, z in [(0.0, 0.0, -0.1), (12.5, 0.3, -0.5), (25.0, -0.9, -1.0)]:
        assert L.gbo_eos(ecp, t, s, z, 1) == grid.eos_np(ec, t, s, z, 1)
        assert L.gbo_eos(ecp, t, s, z, 0) == grid.eos_np(ec, t, s, z, 0)
        dz = C.c_double()
        tec = C.c_double()
        L.gbo_eosd(ecp, t, t + 1.0, s, s + 0.1, z, 3.0, 1, C.byref(dz), C.byref(tec))
        d2, t2 = gnp.eosd(ec, t, t + 1.0, s, s + 0.1, z, 3.0, 1)
        assert (dz.value, tec.value) == (d2, t2)


def test_oracle_rejects_bad_options(oracle):
    import ctypes as C
    from cgenie_gb300.abi import GridRefs, dptr, iptr
    m = grid.make_member(grid.MemberConfig(maxi=6, maxj=5, maxk=4, maxl=2, seed=1))
    r = GridRefs(m)
    r.params.imld = 2
    s = oracle.OracleState(m, refs=r)
    with pytest.raises(RuntimeError):
        s.step(1)
    # imld = 1 needs the wind energy and its decay profile
    r = GridRefs(m)
    r.params.imld = 1
    r.grid.mldketau = None
    s = oracle.OracleState(m, refs=r)
    with pytest.raises(RuntimeError):
        s.step(1)
