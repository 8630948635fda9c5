"""CPU checks of the 2-D surface steppers' restatements: tstipa (src/embm/embm.f90:2039-2138)
and tstipsic (src/goldsteinseaice/gold_seaice.f90:937-1058); the C and NumPy oracles agree
bit for bit, and known-answer properties of the schemes."""
import os

import numpy as np
import pytest

from cgenie_gb300 import grid, surface
from oracle import oracle_lib as ol
from oracle import surface_np as snp


def np_step(c, n):
    snp.step(c.kind, c.maxk, c.dt, c.dphi, c.rdphi, c.betaz, c.betam, c.diffmod0, c.ppmin, c.ppmax, c.diffsic,
             c.tsc, c.rc, c.cv, c.dsv, c.rdsv, c.rds, c.diffa, c.k1, c.tq, c.tq1, c.source, c.vel, c.pptn, n)


CASES = [
    (dict(maxi=12, maxj=10, maxk=8, maxl=2, seed=1), "embm", 3, 0.0),
    (dict(maxi=36, maxj=36, maxk=16, maxl=2, seed=2), "embm", 2, 0.7),   # precipitation-dependent diffusion
    (dict(maxi=37, maxj=23, maxk=8, maxl=2, seed=3), "embm", 1, 0.0),
    (dict(maxi=12, maxj=10, maxk=8, maxl=2, seed=4), "seaice", 1, 0.0),
    (dict(maxi=36, maxj=36, maxk=16, maxl=2, seed=5, land_frac=0.5), "seaice", 1, 0.0),
]


@pytest.mark.parametrize("case", CASES, ids=["embm_small", "embm_diffmod", "embm_odd", "ice_small", "ice_land"])
def test_restatements_agree_bitwise(case):
    cfg, kind, n, dm = case
    m = grid.make_member(grid.MemberConfig(**cfg))
    c = surface.embm_case(m, seed=6, diffmod0=dm) if kind == "embm" else surface.seaice_case(m, seed=6)
    a, b = c.copy(), c.copy()
    ol.surface_step(a, n)
    np_step(b, n)
    assert np.array_equal(a.tq, b.tq) and np.array_equal(a.tq1, b.tq1)
    assert not np.array_equal(a.tq, c.tq)
    if kind == "seaice":
        dry = m.k1[1:-1, 1:-1] > m.maxk
        assert np.array_equal(a.tq[dry], c.tq[dry])      # land cells are not updated
        assert np.array_equal(a.tq1, c.tq1)              # tq1 is left to step_seaice


def test_uniform_field_without_forcing_is_steady():
    """With zero winds and no source a uniform tracer stays uniform to rounding: every face
    flux cie*T(i+1) + ciw*T(i) is then diffusion (cie = -ciw) of a zero gradient."""
    m = grid.make_member(grid.MemberConfig(maxi=12, maxj=10, maxk=8, maxl=2, seed=7))
    c = surface.embm_case(m, seed=8)
    c.vel[...] = 0.0
    c.source[...] = 0.0
    c.tq[..., 0] = 12.5
    c.tq[..., 1] = 0.01
    c.tq1[...] = c.tq
    ol.surface_step(c, 4)
    np.testing.assert_allclose(c.tq[..., 0], 12.5, rtol=1e-13)
    np.testing.assert_allclose(c.tq[..., 1], 0.01, rtol=1e-13)


def test_oracle_header_cites_reference():
    src = open(os.path.join(os.path.dirname(os.path.dirname(os.path.abspath(__file__))), "oracle",
                            "surface_oracle.c")).read()
    assert "ORACLE -- test infrastructure only" in src
    assert "embm.f90:2039-2138" in src and "gold_seaice.f90:937-1058" in src
    assert "parity unpinned" in src


@pytest.mark.parametrize("cfg", [dict(maxi=12, maxj=10, maxk=8, maxl=2, seed=9),
                                 dict(maxi=36, maxj=36, maxk=16, maxl=2, seed=10, land_frac=0.5)])
def test_explicit_seaice_restatements_agree(cfg):
    """tstepsic: the C oracle keeps the reference's west/south flux carries, the NumPy one
    computes whole-array face fluxes; the area/height thresholds stop advection in some cells."""
    m = grid.make_member(grid.MemberConfig(**cfg))
    c = surface.seaice_case(m, seed=11, explicit=True)
    assert (c.tq1[..., 1] > c.sica_thresh).any() and (c.tq1[..., 0] > c.sich_thresh).any()
    a, b = c.copy(), c.copy()
    ol.surface_step(a, 1)
    snp.tstepsic(b.maxk, b.dt, b.rdphi, b.diffsic, b.tsc, b.sica_thresh, b.sich_thresh, b.rc, b.cv, b.rdsv, b.rds,
                 b.k1, b.tq, b.tq1, b.source, b.vel)
    assert np.array_equal(a.tq, b.tq)
    assert not np.array_equal(a.tq, c.tq)


def test_seaice_diag_splits_the_change():
    """tstipsic's diagnostics (gold_seaice.f90:1046-1056): the thermal part is the source
    term's contribution, the dynamical part the rest of the change; land cells keep their
    values."""
    m = grid.make_member(grid.MemberConfig(maxi=36, maxj=36, maxk=16, maxl=2, seed=5, land_frac=0.5))
    c = surface.seaice_case(m, seed=6)
    a = c.copy()
    np_step(a, 1)
    th, dy = np.full_like(c.tq, 7.0), np.full_like(c.tq, 7.0)
    snp.seaice_diag(c.maxk, c.dt, c.tsc, c.k1, a.tq, c.tq1, c.source, th, dy)
    wet = m.k1[1:-1, 1:-1] <= m.maxk
    assert np.array_equal(th[wet], (c.tsc * c.dt * c.source)[wet])
    np.testing.assert_allclose((th + dy)[wet], (a.tq - c.tq1)[wet], rtol=0, atol=1e-12 * np.abs(a.tq).max())
    assert (th[~wet] == 7.0).all() and (dy[~wet] == 7.0).all()
    assert np.abs(dy[wet]).max() > 0


def test_seaice_post_known_answers():
    """step_seaice's post-processing (gold_seaice.f90:599-619) on hand-set cells: area held in
    [0, 1], thin ice removed with its heat and water, varice1 = varice, land untouched."""
    m = grid.make_member(grid.MemberConfig(maxi=12, maxj=10, maxk=8, maxl=2, seed=4, land_frac=0.3))
    c = surface.seaice_case(m, seed=6)
    wet = np.argwhere(m.k1[1:-1, 1:-1] <= m.maxk)
    dry = np.argwhere(m.k1[1:-1, 1:-1] > m.maxk)
    (j0, i0), (j1, i1) = wet[0], wet[1]
    tq = np.zeros_like(c.tq)
    tq[j0, i0] = (0.005, 1.4)    # thin: removed
    tq[j1, i1] = (0.5, -0.2)     # area clamped to 0
    jd, id_ = dry[0]
    tq[jd, id_] = (0.001, 2.0)   # land: untouched
    tq1 = np.full_like(tq, 9.0)
    dtha = np.full_like(tq, 2e-9)
    p = surface.seaice_post_constants(c)
    fx, fw = snp.seaice_post(c.maxk, c.k1, tq, tq1, dtha, p.rhoio, p.rhoice, p.hlf, p.hmin, p.rdtdim, p.m2mm)
    assert tuple(tq[j0, i0]) == (0.0, 0.0) and tuple(tq1[j0, i0]) == (0.0, 0.0)
    assert fx[j0, i0] == -(0.005 * 913.0 * 3.34e5 * p.rdtdim)
    assert fw[j0, i0] == (-(p.rhoio * 2e-9) + 0.005 * p.rhoio * p.rdtdim) * 1000.0
    assert tuple(tq[j1, i1]) == (0.5, 0.0) and fx[j1, i1] == 0.0
    assert fw[j1, i1] == -(p.rhoio * 2e-9) * 1000.0
    assert tuple(tq[jd, id_]) == (0.001, 2.0) and tuple(tq1[jd, id_]) == (9.0, 9.0)
    assert fx[jd, id_] == 0.0 and fw[jd, id_] == 0.0
