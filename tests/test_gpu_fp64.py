"""GPU parity of the plain FP64 form against the oracle, through the C-ABI.

The plain form keeps the reference's operation order with no FMA contraction,
so every comparison here is bit-exact (np.array_equal), including rho, the
convection diagnostics cost/icosd and the isoneutral diagnostics dmax/limps."""
import glob
import os

import numpy as np
import pytest

import member_io
from cgenie_gb300 import abi, grid

pytestmark = pytest.mark.gpu

GOLDEN = sorted(glob.glob(os.path.join(os.path.dirname(__file__), "golden", "*.npz")))


def run_gpu(m, steps, chunks=None, **kw):
    from cgenie_gb300.goldstein import new_member_run
    g = new_member_run(m, **kw)
    for n in (chunks or [steps]):
        g.tstepo(n)
    out = g.download()
    out["inventory"] = g.inventory()
    if g.refs.params.imld == 1:
        out["mld"], out["mldk"] = g.download_mld()
    g.close()
    return out


def assert_same(out, ref, names=("ts", "ts1", "rho", "cost", "icosd")):
    for n in names:
        a, b = out[n], ref[n]
        if not np.array_equal(a, b):
            d = np.abs(np.asarray(a, float) - np.asarray(b, float))
            idx = np.unravel_index(np.argmax(d), d.shape)
            raise AssertionError(f"{n}: {np.count_nonzero(d)} cells differ, max {d.max()} at {idx}")


@pytest.mark.parametrize("path", GOLDEN, ids=[os.path.basename(p)[:-4] for p in GOLDEN])
def test_golden_fixtures_bitexact(gpu_lib, path):
    m, ref = member_io.load(path)
    out = run_gpu(m, int(ref["steps"]))
    assert_same(out, ref)
    if "mld" in ref:
        assert_same(out, ref, ("mld", "mldk"))
    assert out["dmax"] == float(ref["dmax"])
    assert out["limps"] == int(ref["limps"])
    np.testing.assert_allclose(out["inventory"], ref["inventory"], rtol=1e-14)


def oracle_run(oracle, m, steps):
    s = oracle.OracleState(m)
    s.step(steps)
    return dict(ts=s.ts, ts1=s.ts1, rho=s.rho, cost=s.cost, icosd=s.icosd, dmax=s.dmax.value,
                limps=s.limps.value, inventory=s.inventory())


def test_config1_36x36x16_l2_100_steps(gpu_lib, oracle):
    m = grid.make_member(grid.config_c1())
    ref = oracle_run(oracle, m, 100)
    out = run_gpu(m, 100)
    assert_same(out, ref)
    np.testing.assert_allclose(out["inventory"], ref["inventory"], rtol=1e-14)


def test_config2_36x36x16_l17_diso_200_steps(gpu_lib, oracle):
    m = grid.make_member(grid.config_c2())
    ref = oracle_run(oracle, m, 200)
    out = run_gpu(m, 200, chunks=[1, 99, 100])
    assert_same(out, ref)
    assert out["dmax"] == ref["dmax"] and out["limps"] == ref["limps"]


@pytest.mark.parametrize("kw", [
    dict(maxi=37, maxj=23, maxk=13, maxl=5, seed=31, diso=True),                # partial tiles, odd maxk
    dict(maxi=5, maxj=3, maxk=2, maxl=2, seed=32, land_frac=0.0),               # smallest grid
    dict(maxi=8, maxj=6, maxk=64, maxl=3, seed=33, diso=True, noise=1.0),      # deepest supported column
    dict(maxi=6, maxj=5, maxk=7, maxl=128, seed=34, diso=True),                 # most tracers
    dict(maxi=36, maxj=36, maxk=32, maxl=4, seed=35, iconv=1, ieos=1, diso=True, noise=2.0),
    dict(maxi=18, maxj=18, maxk=16, maxl=3, seed=36, iediff=2, ediffpow2=0.7),  # general power
    dict(maxi=18, maxj=18, maxk=16, maxl=3, seed=37, land_frac=0.0, forcing=1.0),
])
def test_shapes_and_branches(gpu_lib, oracle, kw):
    m = grid.make_member(grid.MemberConfig(**kw))
    ref = oracle_run(oracle, m, 6)
    out = run_gpu(m, 6, chunks=[2, 4])
    if kw.get("iediff") and kw.get("ediffpow2") not in (0.0, 0.5, 1.0):
        # the general power uses CUDA's pow (not glibc's): not bit-identical
        for n in ("ts", "ts1"):
            np.testing.assert_allclose(out[n], ref[n], rtol=1e-12, atol=1e-300)
        return
    assert_same(out, ref)
    assert out["dmax"] == ref["dmax"] and out["limps"] == ref["limps"]


def test_download_before_step_returns_upload(gpu_lib):
    from cgenie_gb300.goldstein import new_member_run
    m = grid.make_member(grid.MemberConfig(maxi=12, maxj=10, maxk=8, maxl=3, seed=41))
    m.ts1[...] = m.ts + 1.0   # distinct ts/ts1, land and halos included
    g = new_member_run(m)
    out = g.download()
    assert np.array_equal(out["ts"], m.ts) and np.array_equal(out["ts1"], m.ts1)
    assert np.array_equal(out["rho"], m.rho)
    g.close()


def test_distinct_ts_ts1_upload_matches_oracle(gpu_lib, oracle):
    """ts and ts1 may differ on upload (land, halos, forcing slot): the step reads
    ts1 and the forcing slot of ts exactly as the reference does."""
    m = grid.make_member(grid.MemberConfig(maxi=12, maxj=10, maxk=8, maxl=3, seed=42, diso=True, forcing=1.0))
    rng = np.random.default_rng(0)
    m.ts1[...] = m.ts + 1e-3 * rng.standard_normal(m.ts.shape)
    ref = oracle_run(oracle, m, 3)
    out = run_gpu(m, 3)
    assert_same(out, ref)


def test_forcing_update_between_steps(gpu_lib, oracle):
    from cgenie_gb300.goldstein import new_member_run
    m = grid.make_member(grid.MemberConfig(maxi=12, maxj=10, maxk=8, maxl=2, seed=43))
    s = oracle.OracleState(m)
    g = new_member_run(m)
    rng = np.random.default_rng(1)
    for step in range(4):
        top = np.zeros((m.maxj + 2, m.maxi + 2, m.maxl))
        top[1:-1, 1:-1] = 1e-3 * rng.standard_normal((m.maxj, m.maxi, m.maxl))
        s.ts[m.maxk + 1] = top
        g.set_forcing(top)
        s.step(1)
        g.tstepo(1)
    out = g.download()
    assert np.array_equal(out["ts"], s.ts) and np.array_equal(out["ts1"], s.ts1)
    g.close()


def test_error_codes(gpu_lib):
    from cgenie_gb300.goldstein import Goldstein, GoldsteinError
    m = grid.make_member(grid.MemberConfig(maxi=6, maxj=5, maxk=4, maxl=2, seed=44))
    g = Goldstein(m)
    with pytest.raises(GoldsteinError) as e:
        g.tstepo(1)
    assert e.value.code == abi.GB_GO_ENOTREADY
    g.close()
    bad = grid.make_member(grid.MemberConfig(maxi=6, maxj=5, maxk=4, maxl=2, seed=45))
    bad.k1[2, 0] = bad.k1[2, bad.maxi] + 1 if bad.k1[2, bad.maxi] < 5 else 1
    with pytest.raises(GoldsteinError) as e:
        Goldstein(bad)
    assert e.value.code == abi.GB_GO_EINVAL
    import ctypes as C
    from cgenie_gb300.abi import GridRefs
    h = C.c_void_p()
    # the mixed layer: imld is 0 or 1; imld = 1 needs its inputs
    r = GridRefs(m)
    r.params.imld = 2
    assert gpu_lib.gb_go_create(C.byref(r.dims), C.byref(r.params), C.byref(r.grid), -1,
                                C.byref(h)) == abi.GB_GO_EINVAL
    r = GridRefs(m, imld=1)
    r.grid.mldketau = None
    assert gpu_lib.gb_go_create(C.byref(r.dims), C.byref(r.params), C.byref(r.grid), -1,
                                C.byref(h)) == abi.GB_GO_EINVAL
    r = GridRefs(m)
    r.params.ieos = 3
    assert gpu_lib.gb_go_create(C.byref(r.dims), C.byref(r.params), C.byref(r.grid), -1,
                                C.byref(h)) == abi.GB_GO_EINVAL


def test_conservation_1000_steps(gpu_lib):
    """Zero forcing: the compensated inventory drifts by rounding only."""
    from cgenie_gb300.goldstein import new_member_run
    m = grid.make_member(grid.config_c2())
    g = new_member_run(m)
    inv0 = g.inventory()
    g.tstepo(1000)
    inv1 = g.inventory()
    rel = np.abs(inv1 - inv0) / np.abs(inv0)
    assert np.all(rel < 1e-12), rel
    g.close()


def test_kernel_launches_counted(gpu_lib):
    from cgenie_gb300.goldstein import kernel_launch_count, new_member_run
    m = grid.make_member(grid.MemberConfig(maxi=6, maxj=5, maxk=4, maxl=2, seed=46))
    g = new_member_run(m)
    n0 = kernel_launch_count()
    g.tstepo(5)
    g.sync()
    assert kernel_launch_count() - n0 == 5
    g.close()
