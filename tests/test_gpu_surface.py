"""GPU parity of the 2-D surface steppers (tstipa, src/embm/embm.f90:2039-2138; tstipsic,
src/goldsteinseaice/gold_seaice.f90:937-1058) against the C oracle, through the C-ABI
(include/gb_embm.h).  The device keeps the reference's operation order without FMA
contraction: every comparison is bit-exact."""
import numpy as np
import pytest

from cgenie_gb300 import abi, grid, surface
from oracle import oracle_lib as ol

pytestmark = pytest.mark.gpu


def run(c, nsteps, calls=1):
    s = surface.SurfaceStepper(c)
    s.upload_state()
    s.set_forcing()
    for _ in range(calls):
        s.step(nsteps)
    out = s.download()
    s.close()
    return out


@pytest.mark.parametrize("cfg,kind,nsteps,calls,dm", [
    (dict(maxi=12, maxj=10, maxk=8, maxl=2, seed=11), "embm", 1, 1, 0.0),
    (dict(maxi=36, maxj=36, maxk=16, maxl=2, seed=12), "embm", 5, 2, 0.0),     # 10 steps, two launches
    (dict(maxi=36, maxj=36, maxk=16, maxl=2, seed=13), "embm", 3, 1, 0.7),     # pptn-dependent diffusion
    (dict(maxi=37, maxj=23, maxk=8, maxl=2, seed=14), "embm", 2, 1, 0.0),      # odd shape
    (dict(maxi=64, maxj=64, maxk=8, maxl=2, seed=15), "embm", 2, 1, 0.0),      # 8 blocks of 8 rows per tracer
    (dict(maxi=128, maxj=61, maxk=8, maxl=2, seed=21), "embm", 2, 1, 0.0),     # ragged last block (5 rows)
    (dict(maxi=180, maxj=90, maxk=8, maxl=2, seed=22, land_frac=0.4), "seaice", 1, 1, 0.0),   # 16,200 cells
    (dict(maxi=1, maxj=2, maxk=4, maxl=2, seed=16, land_frac=0.0), "embm", 2, 1, 0.0),   # smallest grid
    (dict(maxi=12, maxj=10, maxk=8, maxl=2, seed=17), "seaice", 1, 1, 0.0),
    (dict(maxi=36, maxj=36, maxk=16, maxl=2, seed=18, land_frac=0.5), "seaice", 1, 3, 0.0),
    (dict(maxi=36, maxj=36, maxk=16, maxl=2, seed=23, land_frac=0.5), "ice_explicit", 1, 2, 0.0),
    (dict(maxi=37, maxj=23, maxk=8, maxl=2, seed=24, land_frac=0.0), "ice_explicit", 1, 1, 0.0),
], ids=["embm_small", "embm_10steps", "embm_diffmod", "embm_odd", "embm_64x64", "embm_128x61", "ice_180x90",
        "embm_1x2", "ice_small", "ice_land_3calls", "ice_explicit_land", "ice_explicit_odd"])
def test_bitexact_vs_oracle(gpu_lib, cfg, kind, nsteps, calls, dm):
    m = grid.make_member(grid.MemberConfig(**cfg))
    if kind == "embm":
        c = surface.embm_case(m, seed=3, diffmod0=dm)
    else:
        c = surface.seaice_case(m, seed=3, explicit=kind == "ice_explicit")
    tq, tq1 = run(c.copy(), nsteps, calls)
    ref = c.copy()
    for _ in range(calls):
        ol.surface_step(ref, nsteps)
    assert np.array_equal(tq, ref.tq), np.abs(tq - ref.tq).max()
    assert np.array_equal(tq1, ref.tq1)


def test_errors(gpu_lib):
    from cgenie_gb300.goldstein import GoldsteinError
    m = grid.make_member(grid.MemberConfig(maxi=12, maxj=10, maxk=8, maxl=2, seed=19))
    c = surface.seaice_case(m, seed=4)
    s = surface.SurfaceStepper(c)
    with pytest.raises(GoldsteinError) as e:
        s.step(1)
    assert e.value.code == abi.GB_GO_ENOTREADY
    s.upload_state()
    s.set_forcing()
    with pytest.raises(GoldsteinError) as e:
        s.step(2)                 # sea ice: one step per call
    assert e.value.code == abi.GB_GO_EINVAL
    s.close()
    big = grid.make_member(grid.MemberConfig(maxi=200, maxj=200, maxk=8, maxl=2, seed=20))   # 40,000 cells
    with pytest.raises(GoldsteinError) as e:
        surface.SurfaceStepper(surface.embm_case(big, seed=5))
    assert e.value.code == abi.GB_GO_ERANGE
    # sea ice needs land in rows 0 and maxj+1 (nothing may read beyond row maxj)
    c = surface.seaice_case(m, seed=6)
    c.k1 = c.k1.copy()
    c.k1[-1, 3] = 1
    with pytest.raises(GoldsteinError) as e:
        surface.SurfaceStepper(c)
    assert e.value.code == abi.GB_GO_EINVAL


@pytest.mark.parametrize("kind", ["embm", "ice_explicit", "ice"])
def test_step_many_bitexact(gpu_lib, kind):
    """Several grids of one shape (distinct masks, states and forcing) in one launch."""
    cases = []
    for n in range(5):
        m = grid.make_member(grid.MemberConfig(maxi=36, maxj=36, maxk=8, maxl=2, seed=60 + n, land_frac=0.3))
        if kind == "embm":
            cases.append(surface.embm_case(m, seed=70 + n))
        else:
            cases.append(surface.seaice_case(m, seed=70 + n, explicit=kind == "ice_explicit"))
    steppers = [surface.SurfaceStepper(c.copy()) for c in cases]
    for s in steppers:
        s.upload_state()
        s.set_forcing()
    nsteps = 3 if kind == "embm" else 1
    surface.step_many(steppers, nsteps)
    for s, c in zip(steppers, cases):
        tq, tq1 = s.download()
        ref = c.copy()
        ol.surface_step(ref, nsteps)
        assert np.array_equal(tq, ref.tq) and np.array_equal(tq1, ref.tq1)
        s.close()


def test_step_many_rejects_mixed_shapes(gpu_lib):
    from cgenie_gb300.goldstein import GoldsteinError
    a = surface.SurfaceStepper(surface.embm_case(grid.make_member(grid.MemberConfig(maxi=12, maxj=10, maxk=4, maxl=2, seed=1)), seed=1))
    b = surface.SurfaceStepper(surface.embm_case(grid.make_member(grid.MemberConfig(maxi=14, maxj=10, maxk=4, maxl=2, seed=2)), seed=2))
    for s in (a, b):
        s.upload_state()
        s.set_forcing()
    with pytest.raises(GoldsteinError) as e:
        surface.step_many([a, b], 1)
    assert e.value.code == abi.GB_GO_EINVAL
    a.close()
    b.close()


@pytest.mark.parametrize("cfg", [dict(maxi=36, maxj=36, maxk=16, maxl=2, seed=25, land_frac=0.5),
                                 dict(maxi=180, maxj=90, maxk=8, maxl=2, seed=26, land_frac=0.4)],
                         ids=["36x36", "180x90"])
def test_seaice_diagnostics_bitexact(gpu_lib, cfg):
    """variceth / varicedy of tstipsic (gold_seaice.f90:1046-1056) against the NumPy oracle,
    over two calls (the second starts from the first's ice, with new forcing); land cells stay 0."""
    from oracle import surface_np as snp
    m = grid.make_member(grid.MemberConfig(**cfg))
    c = surface.seaice_case(m, seed=8)
    s = surface.SurfaceStepper(c.copy())
    ref = c.copy()
    th_ref, dy_ref = np.zeros_like(c.tq), np.zeros_like(c.tq)
    rng = np.random.default_rng(9)
    for call in range(2):
        if call:
            ref.tq1 = ref.tq.copy()
            ref.source = ref.source * rng.uniform(0.5, 1.5, ref.source.shape)
        s.upload_state(ref.tq, ref.tq1)
        s.set_forcing(source=ref.source)
        s.step(1)
        tq1_before = ref.tq1.copy()
        ol.surface_step(ref, 1)
        snp.seaice_diag(ref.maxk, ref.dt, ref.tsc, ref.k1, ref.tq, tq1_before, ref.source, th_ref, dy_ref)
        th, dy = s.download_seaice_diag()
        assert np.array_equal(th.view(np.uint64), th_ref.view(np.uint64))
        assert np.array_equal(dy.view(np.uint64), dy_ref.view(np.uint64))
    dry = m.k1[1:-1, 1:-1] > m.maxk
    assert dry.any() and not th[dry].any() and not dy[dry].any()
    assert np.abs(dy).max() > 0 and np.abs(th).max() > 0
    s.close()


def test_seaice_diagnostics_forms(gpu_lib):
    """The explicit step leaves the diagnostics at 0 (tstepsic does not set them); batched
    implicit steps set each grid's own; an EMBM handle has none."""
    from cgenie_gb300.goldstein import GoldsteinError
    from oracle import surface_np as snp
    m = grid.make_member(grid.MemberConfig(maxi=36, maxj=36, maxk=8, maxl=2, seed=27, land_frac=0.3))
    s = surface.SurfaceStepper(surface.seaice_case(m, seed=10, explicit=True))
    s.upload_state()
    s.set_forcing()
    s.step(1)
    th, dy = s.download_seaice_diag()
    assert not th.any() and not dy.any()
    s.close()
    cases = [surface.seaice_case(grid.make_member(grid.MemberConfig(maxi=36, maxj=36, maxk=8, maxl=2, seed=80 + n,
                                                                    land_frac=0.3)), seed=90 + n) for n in range(3)]
    steppers = [surface.SurfaceStepper(c.copy()) for c in cases]
    for st in steppers:
        st.upload_state()
        st.set_forcing()
    surface.step_many(steppers, 1)
    for st, c in zip(steppers, cases):
        ref = c.copy()
        ol.surface_step(ref, 1)
        th_ref, dy_ref = np.zeros_like(c.tq), np.zeros_like(c.tq)
        snp.seaice_diag(c.maxk, c.dt, c.tsc, c.k1, ref.tq, c.tq1, c.source, th_ref, dy_ref)
        th, dy = st.download_seaice_diag()
        assert np.array_equal(th, th_ref) and np.array_equal(dy, dy_ref)
        st.close()
    e_ = surface.SurfaceStepper(surface.embm_case(m, seed=11))
    with pytest.raises(GoldsteinError) as e:
        e_.download_seaice_diag()
    assert e.value.code == abi.GB_GO_EINVAL
    e_.close()


def _post_case(m, seed, explicit):
    """A sea-ice case with thin ice (under hmin) and areas above 1 on some ocean cells."""
    c = surface.seaice_case(m, seed=seed, explicit=explicit)
    rng = np.random.default_rng(seed + 1)
    thin = rng.random(c.tq.shape[:2]) < 0.2
    c.tq[..., 0] = np.where(thin, c.tq[..., 0] * 0.003, c.tq[..., 0])
    c.tq[..., 1] = np.where(rng.random(c.tq.shape[:2]) < 0.1, c.tq[..., 1] + 0.3, c.tq[..., 1])
    c.tq1 = c.tq.copy()
    return c


def _ref_post_steps(c, nsteps, post):
    """nsteps step_seaice steps on the oracles: transport, diagnostics, post-processing."""
    from oracle import surface_np as snp
    ref = c.copy()
    th, dy = np.zeros_like(c.tq), np.zeros_like(c.tq)
    fx = fw = None
    for _ in range(nsteps):
        before = ref.tq1.copy()
        ol.surface_step(ref, 1)
        if ref.kind == abi.GB_EA_SEAICE:
            snp.seaice_diag(ref.maxk, ref.dt, ref.tsc, ref.k1, ref.tq, before, ref.source, th, dy)
        fx, fw = snp.seaice_post(ref.maxk, ref.k1, ref.tq, ref.tq1, ref.source, post.rhoio, post.rhoice, post.hlf,
                                 post.hmin, post.rdtdim, post.m2mm)
    return ref, th, dy, fx, fw


def _bits_equal(a, b):
    return np.array_equal(np.asarray(a).view(np.uint64), np.asarray(b).view(np.uint64))


@pytest.mark.parametrize("explicit", [False, True], ids=["tstipsic", "tstepsic"])
@pytest.mark.parametrize("cfg", [dict(maxi=36, maxj=36, maxk=16, maxl=2, seed=28, land_frac=0.5),
                                 dict(maxi=180, maxj=90, maxk=8, maxl=2, seed=29, land_frac=0.4)],
                         ids=["36x36", "180x90"])
def test_seaice_post_steps_bitexact(gpu_lib, cfg, explicit):
    """Several step_seaice steps in one call (transport + gold_seaice.f90:599-619 on the device)
    against the oracles step by step: ice, fluxes and diagnostics bit for bit."""
    m = grid.make_member(grid.MemberConfig(**cfg))
    c = _post_case(m, 30, explicit)
    post = surface.seaice_post_constants(c)
    s = surface.SurfaceStepper(c.copy())
    s.set_seaice_post(post)
    s.upload_state()
    s.set_forcing()
    s.step(3)
    tq, tq1 = s.download()
    fx, fw = s.download_seaice_fluxes()
    th, dy = s.download_seaice_diag()
    s.close()
    ref, th_ref, dy_ref, fx_ref, fw_ref = _ref_post_steps(c, 3, post)
    assert _bits_equal(tq, ref.tq) and _bits_equal(tq1, ref.tq1)
    assert _bits_equal(fx, fx_ref) and _bits_equal(fw, fw_ref)
    assert _bits_equal(th, th_ref) and _bits_equal(dy, dy_ref)
    wet = m.k1[1:-1, 1:-1] <= m.maxk
    assert (fx[wet] != 0).any() and (fw[wet] != 0).any() and not fx[~wet].any() and not fw[~wet].any()
    assert (tq[..., 1] <= 1.0).all() and (tq[..., 1] >= 0.0).all()


def test_seaice_post_many_and_errors(gpu_lib):
    """Batched post-processed steps equal the oracles per grid; grids that differ in
    post-processing cannot step together; EMBM has none; without it sea ice takes one step."""
    from cgenie_gb300.goldstein import GoldsteinError
    cases = [_post_case(grid.make_member(grid.MemberConfig(maxi=36, maxj=36, maxk=8, maxl=2, seed=40 + n,
                                                           land_frac=0.3)), 50 + n, False) for n in range(3)]
    post = surface.seaice_post_constants(cases[0])
    steppers = [surface.SurfaceStepper(c.copy()) for c in cases]
    for st in steppers:
        st.set_seaice_post(post)
        st.upload_state()
        st.set_forcing()
    surface.step_many(steppers, 2)
    for st, c in zip(steppers, cases):
        ref, _, _, fx_ref, fw_ref = _ref_post_steps(c, 2, post)
        tq, tq1 = st.download()
        fx, fw = st.download_seaice_fluxes()
        assert _bits_equal(tq, ref.tq) and _bits_equal(tq1, ref.tq1)
        assert _bits_equal(fx, fx_ref) and _bits_equal(fw, fw_ref)
    steppers[1].set_seaice_post(None)
    with pytest.raises(GoldsteinError) as e:
        surface.step_many(steppers, 1)
    assert e.value.code == abi.GB_GO_EINVAL
    with pytest.raises(GoldsteinError) as e:
        steppers[1].step(2)
    assert e.value.code == abi.GB_GO_EINVAL
    for st in steppers:
        st.close()
    m = grid.make_member(grid.MemberConfig(maxi=12, maxj=10, maxk=8, maxl=2, seed=41))
    e_ = surface.SurfaceStepper(surface.embm_case(m, seed=1))
    with pytest.raises(GoldsteinError) as e:
        e_.set_seaice_post(post)
    assert e.value.code == abi.GB_GO_EINVAL
    with pytest.raises(GoldsteinError) as e:
        e_.download_seaice_fluxes()
    assert e.value.code == abi.GB_GO_EINVAL
    e_.close()
