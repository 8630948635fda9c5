"""GPU parity of the BIOGEM tracer coupling (src/biogem/biogem.f90:1885-2077) against the C
oracle, through the C-ABI (include/gb_biogem.h).  The device path keeps the reference's
operation order (column sums left to right, no FMA contraction): every comparison is
bit-exact."""
import numpy as np
import pytest

from cgenie_gb300 import abi, biogem, grid
from oracle import oracle_lib as ol

pytestmark = pytest.mark.gpu


def device_run(m, st, *, steps_before=0, steps_after=0, force=False, couplings=1, st2=None):
    from cgenie_gb300.goldstein import new_member_run
    g = new_member_run(m)
    bg = biogem.BiogemCoupling(m, n_l_sed=st.vbio_part.shape[-1], force_ts=force)
    bg.upload(st)
    bg.set_increments(st)
    if steps_before:
        g.tstepo(steps_before)
    bg.tracercoupling(g)
    for c in range(1, couplings):
        g.tstepo(3)
        bg.set_increments(st2)
        bg.tracercoupling(g)
    if steps_after:
        g.tstepo(steps_after)
    out = g.download()
    out["bg"] = bg.download()
    bg.close()
    g.close()
    return out


def oracle_run(m, st, *, steps_before=0, steps_after=0, force=False, couplings=1, st2=None):
    s = ol.OracleState(m)
    a = st.copy()
    if steps_before:
        s.step(steps_before)
    go, go1 = ol.bg_tracercoupling(m, a, ol.go_ts_interior(s.ts), force_ts=force)
    ol.after_coupling(s, go, go1)
    for c in range(1, couplings):
        s.step(3)
        a.vdocn, a.vdbio_part = st2.vdocn, st2.vdbio_part
        go, go1 = ol.bg_tracercoupling(m, a, ol.go_ts_interior(s.ts), force_ts=force)
        ol.after_coupling(s, go, go1)
    if steps_after:
        s.step(steps_after)
    return s, a


def assert_bitexact(out, s, a):
    for name in ("ts", "ts1", "rho"):
        x, y = out[name], getattr(s, name)
        if not np.array_equal(x, y):
            d = np.abs(x - y)
            raise AssertionError(f"{name}: {np.count_nonzero(d)} cells differ, max {d.max()}")
    vocn, mass, rmass, vbio = out["bg"]
    assert np.array_equal(vocn, a.vocn)
    assert np.array_equal(mass, a.mass)
    assert np.array_equal(rmass, a.rmass)
    assert np.array_equal(vbio, a.vbio_part)


@pytest.mark.parametrize("kw", [
    dict(cfg=dict(maxi=12, maxj=10, maxk=8, maxl=5, seed=21), n_l_sed=3, force=False),
    dict(cfg=dict(maxi=12, maxj=10, maxk=8, maxl=5, seed=22), n_l_sed=3, force=True),
    dict(cfg=dict(maxi=7, maxj=5, maxk=4, maxl=2, seed=23), n_l_sed=0, force=False),
    dict(cfg=dict(maxi=36, maxj=36, maxk=16, maxl=17, seed=24, diso=True), n_l_sed=8, force=False),
    dict(cfg=dict(maxi=8, maxj=6, maxk=64, maxl=3, seed=25), n_l_sed=1, force=True),
    dict(cfg=dict(maxi=6, maxj=5, maxk=7, maxl=128, seed=26), n_l_sed=2, force=False),
], ids=["small", "force_ts", "ts_only", "36x36x16_l17", "deepest", "most_tracers"])
def test_coupling_after_upload_bitexact(gpu_lib, kw):
    m = grid.make_member(grid.MemberConfig(**kw["cfg"]))
    st = biogem.make_state(m, n_l_sed=kw["n_l_sed"], seed=7)
    out = device_run(m, st, force=kw["force"])
    s, a = oracle_run(m, st, force=kw["force"])
    assert_bitexact(out, s, a)


def test_steps_coupling_steps_bitexact(gpu_lib):
    """tstepo x 5, coupling, tstepo x 3, coupling with new increments, tstepo x 4: the device
    state after each coupling continues exactly as step_goldstein's copy-in leaves it."""
    m = grid.make_member(grid.MemberConfig(maxi=18, maxj=14, maxk=12, maxl=6, seed=27, diso=True, iconv=1,
                                           ieos=1, noise=2.0))
    st = biogem.make_state(m, n_l_sed=2, seed=8)
    st2 = biogem.make_state(m, n_l_sed=2, seed=9)
    out = device_run(m, st, steps_before=5, steps_after=4, couplings=2, st2=st2)
    s, a = oracle_run(m, st, steps_before=5, steps_after=4, couplings=2, st2=st2)
    assert_bitexact(out, s, a)


def test_zero_inventory_tracer(gpu_lib):
    """A tracer whose inventory is 0 takes rtot_new = 0 (biogem.f90:1991-1995)."""
    m = grid.make_member(grid.MemberConfig(maxi=12, maxj=10, maxk=8, maxl=5, seed=28))
    m.ts[..., 3] = 0.0
    m.ts1[..., 3] = 0.0
    st = biogem.make_state(m, n_l_sed=1, seed=10)
    st.vocn[..., 3] = 0.0
    st.vdocn[..., 3] = 0.0
    out = device_run(m, st)
    s, a = oracle_run(m, st)
    assert_bitexact(out, s, a)
    assert np.all(out["bg"][0][..., 3] == 0.0)


def test_config5_grid_bitexact(gpu_lib):
    """360x180x32, 24 tracers: the column sums run over ~45,000 columns."""
    m = grid.make_member(grid.config_c5())
    st = biogem.make_state(m, n_l_sed=8, seed=11)
    out = device_run(m, st)
    s, a = oracle_run(m, st)
    assert_bitexact(out, s, a)


def test_errors(gpu_lib):
    from cgenie_gb300.goldstein import GoldsteinError, new_member_run
    m = grid.make_member(grid.MemberConfig(maxi=12, maxj=10, maxk=8, maxl=4, seed=29))
    st = biogem.make_state(m, n_l_sed=1, seed=12)
    g = new_member_run(m)
    bg = biogem.BiogemCoupling(m, n_l_sed=1)
    with pytest.raises(GoldsteinError) as e:
        bg.tracercoupling(g)
    assert e.value.code == abi.GB_GO_ENOTREADY
    bg.upload(st)
    bg.set_increments(st)
    other = grid.make_member(grid.MemberConfig(maxi=12, maxj=10, maxk=8, maxl=5, seed=30))
    g2 = new_member_run(other)
    with pytest.raises(GoldsteinError) as e:
        bg.tracercoupling(g2)
    assert e.value.code == abi.GB_GO_EINVAL
    for h in (g, g2):
        h.close()
    bg.close()


def test_split_precision_handle(gpu_lib):
    """The coupling on a split-precision handle: its state is exported, coupled in FP64 and
    re-imported; steps before and after stay within the form's bars of the oracle (T and S
    1e-11, the other tracers 1e-6), BIOGEM's fields within 1e-10."""
    from cgenie_gb300.goldstein import new_member_run
    m = grid.make_member(grid.MemberConfig(maxi=18, maxj=14, maxk=12, maxl=6, seed=32, tracer_kind="bgc"))
    st = biogem.make_state(m, n_l_sed=2, seed=14)
    g = new_member_run(m, precision=abi.GB_GO_FP32FLUX)
    bg = biogem.BiogemCoupling(m, n_l_sed=2)
    bg.upload(st)
    bg.set_increments(st)
    g.tstepo(4)
    bg.tracercoupling(g)
    g.tstepo(3)
    out = g.download()
    vocn = bg.download()[0]
    s, a = oracle_run(m, st, steps_before=4, steps_after=3)
    kk = np.arange(m.maxk + 2)[:, None, None]
    wet = (kk >= m.k1[None]) & (kk >= 1) & (kk <= m.maxk)
    wet[:, :, 0] = wet[:, :, -1] = False
    for l in range(m.maxl):
        x, y = out["ts"][..., l][wet], s.ts[..., l][wet]
        err = np.abs(x - y).max() / np.abs(y).max()
        assert err <= (1e-11 if l < 2 else 1e-6), (l, err)
    np.testing.assert_allclose(vocn, a.vocn, rtol=1e-10, atol=1e-12 * np.abs(a.vocn).max())
    bg.close()
    g.close()


def test_reupload_between_couplings(gpu_lib):
    """Dry interior cells are zeroed by the first coupling after each upload: upload a state
    whose dry cells are not 0, couple, upload it again, couple again."""
    from cgenie_gb300.goldstein import new_member_run
    m = grid.make_member(grid.MemberConfig(maxi=12, maxj=10, maxk=8, maxl=4, seed=31))
    kk = np.arange(m.maxk + 2)[:, None, None]
    dry = (kk < m.k1[None]) & (kk >= 1) & (kk <= m.maxk)
    dry[:, 0, :] = dry[:, -1, :] = False
    dry[:, :, 0] = dry[:, :, -1] = False
    m.ts[dry] = 7.0
    m.ts1[dry] = 5.0
    st = biogem.make_state(m, n_l_sed=1, seed=13)
    g = new_member_run(m)
    bg = biogem.BiogemCoupling(m, n_l_sed=1)
    bg.upload(st)
    bg.set_increments(st)
    bg.tracercoupling(g)
    g.upload_state()
    bg.tracercoupling(g)
    out = g.download()
    out["bg"] = bg.download()
    bg.close()
    g.close()
    a = st.copy()
    s = ol.OracleState(m)
    go, go1 = ol.bg_tracercoupling(m, a, ol.go_ts_interior(s.ts))
    s = ol.OracleState(m)
    go, go1 = ol.bg_tracercoupling(m, a, ol.go_ts_interior(s.ts))
    ol.after_coupling(s, go, go1)
    assert_bitexact(out, s, a)
    assert np.all(out["ts"][dry] == 0.0) and np.all(out["ts1"][dry] == 0.0)
