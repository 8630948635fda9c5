"""CPU checks of the BIOGEM tracer coupling restatements (src/biogem/biogem.f90:1885-2077):
the C and NumPy oracles agree bit for bit, and known-answer properties of the routine."""
import numpy as np
import pytest

from cgenie_gb300 import biogem, grid
from oracle import biogem_np as bnp
from oracle import oracle_lib as ol


def np_coupling(m, st, go, force):
    g = np.ascontiguousarray(go.transpose(3, 2, 1, 0))   # [l, i, j, k]
    k1 = m.k1[1:-1, 1:-1].T
    o, o1 = bnp.tracercoupling(g, st.vocn, st.mass, st.volume, st.rmass, st.vdocn, st.vbio_part, st.vdbio_part,
                               k1, (biogem.CONST_ZEROC, biogem.SALN0), force)
    return o.transpose(3, 2, 1, 0), o1.transpose(3, 2, 1, 0)


CASES = [
    dict(cfg=dict(maxi=12, maxj=10, maxk=8, maxl=5, seed=1), n_l_sed=3, force=False),
    dict(cfg=dict(maxi=12, maxj=10, maxk=8, maxl=5, seed=2), n_l_sed=3, force=True),
    dict(cfg=dict(maxi=7, maxj=5, maxk=4, maxl=2, seed=3), n_l_sed=0, force=False),     # T and S only
    dict(cfg=dict(maxi=18, maxj=14, maxk=16, maxl=9, seed=4, land_frac=0.0), n_l_sed=1, force=True),
]


@pytest.mark.parametrize("case", CASES, ids=["plain", "force_ts", "ts_only", "no_land"])
def test_restatements_agree_bitwise(case):
    m = grid.make_member(grid.MemberConfig(**case["cfg"]))
    st = biogem.make_state(m, n_l_sed=case["n_l_sed"], seed=5)
    if m.maxl > 3:
        st.vocn[..., 3] = 0.0          # a tracer with no inventory: rtot_new = 0 (biogem.f90:1991-1995)
        st.vdocn[..., 3] = 0.0
    go = ol.go_ts_interior(m.ts)
    if m.maxl > 3:
        go[..., 3] = 0.0
    a, b = st.copy(), st.copy()
    t, t1 = ol.bg_tracercoupling(m, a, go, force_ts=case["force"])
    u, u1 = np_coupling(m, b, go, case["force"])
    assert np.array_equal(t, u) and np.array_equal(t1, u1) and np.array_equal(t, t1)
    for name in ("vocn", "mass", "rmass", "vbio_part"):
        assert np.array_equal(getattr(a, name), getattr(b, name)), name
    if m.maxl > 3:
        assert np.all(a.vocn[..., 3] == 0.0)


def test_zero_increments_conserve_inventories_and_salinity():
    """With no increments and GOLDSTEIN tracers equal to BIOGEM's (less the offsets), the mean
    salinity is unchanged (s_ratio = 1, masses unchanged), each biogeochemical inventory
    sum(vocn*M) is restored to its old value, and go_ts comes back to rounding."""
    m = grid.make_member(grid.MemberConfig(maxi=18, maxj=14, maxk=12, maxl=6, seed=11))
    st = biogem.make_state(m, n_l_sed=2, seed=12, increments=0.0)
    go = ol.go_ts_interior(m.ts)
    # go_ts consistent with vocn: the biogeochemical tracers salinity-normalised
    cols = biogem.wet_columns(m.k1[1:-1, 1:-1], m.maxk)
    wet = np.zeros(st.mass.shape, bool)
    for n, (_, _, kk) in enumerate(cols):
        wet[n, kk - 1:] = True
    inv0 = [(st.vocn[..., l] * st.mass)[wet].sum() for l in range(2, m.maxl)]
    mass0 = st.mass.copy()
    a = st.copy()
    t, _ = ol.bg_tracercoupling(m, a, go)
    assert np.array_equal(a.mass, mass0)
    inv1 = [(a.vocn[..., l] * a.mass)[wet].sum() for l in range(2, m.maxl)]
    np.testing.assert_allclose(inv1, inv0, rtol=1e-13)
    kk = np.arange(1, m.maxk + 1)[:, None, None]
    w = kk >= m.k1[None, 1:-1, 1:-1]
    np.testing.assert_allclose(t[w], go[w], rtol=1e-13, atol=1e-12)
    assert np.all(t[~w] == 0.0)


def test_column_order_is_i_outer_j_inner():
    k1 = np.array([[1, 9], [2, 1]])   # [j, i] with n_k = 8: column (i=1, j=0) is land
    assert biogem.wet_columns(k1, 8) == [(0, 0, 1), (0, 1, 2), (1, 1, 1)]
    assert bnp.columns(k1.T, 8) == [(0, 0, 1), (0, 1, 2), (1, 1, 1)]


def test_oracle_header_cites_reference():
    import os
    src = open(os.path.join(os.path.dirname(os.path.dirname(os.path.abspath(__file__))), "oracle",
                            "biogem_oracle.c")).read()
    assert "ORACLE -- test infrastructure only" in src
    assert "biogem.f90:1885-2077" in src
    assert "parity unpinned" in src
