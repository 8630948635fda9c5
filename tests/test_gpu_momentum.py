"""GPU parity of the momentum step (wind, jbar, ubarsolv, island, velc of
src/goldstein/goldstein.f90 and goldstein_lib.f90) against the C oracle, through the C-ABI
(include/gb_momentum.h).  The device forms the streamfunction as inverse x right-hand side
instead of the reference's serial back substitution, so psi, ub and u agree to a relative
1e-9 (of each field's largest magnitude), not bit for bit."""
import numpy as np
import pytest

from cgenie_gb300 import abi, grid, momentum
from oracle import oracle_lib as ol

pytestmark = pytest.mark.gpu

RTOL = 1e-9


def close(a, b, name):
    scale = max(np.abs(b).max(), 1e-300)
    err = np.abs(a - b).max() / scale
    assert err <= RTOL, f"{name}: {err:.2e}"


@pytest.mark.parametrize("cfg", [
    dict(maxi=18, maxj=14, maxk=8, maxl=2, seed=51, mask="basin"),
    dict(maxi=18, maxj=14, maxk=8, maxl=2, seed=52, mask="basin_island"),
    dict(maxi=36, maxj=36, maxk=16, maxl=2, seed=53, mask="basin_island"),
    dict(maxi=37, maxj=23, maxk=12, maxl=2, seed=54, mask="basin_island"),
], ids=["18x14", "18x14_island", "36x36_island", "37x23_island"])
@pytest.mark.parametrize("solver", [0, 1], ids=["inverse", "blocktridiag"])
def test_momentum_step_matches_oracle(gpu_lib, cfg, solver):
    from cgenie_gb300.goldstein import new_member_run
    m = grid.make_member(grid.MemberConfig(**cfg))
    c = momentum.make_case(m, seed=5)
    g = new_member_run(m)
    mo = momentum.Momentum(c, solver=solver)
    mo.set_wind()
    o = ol.OracleMomentum(c)
    for _ in range(3):                # three steps on the same density: u1 relaxation enters
        mo.step(g)
        o.step(m.rho)
    out, ref = mo.download(), o.state()
    for n in ("psi", "ub", "u", "u1"):
        close(out[n], ref[n], n)
    mo.close()
    g.close()


@pytest.mark.parametrize("shape", [(128, 72), (360, 180)], ids=["128x72", "360x180"])
def test_large_grid_block_tridiagonal_matches_oracle(gpu_lib, shape):
    """Grids above GB_MO_MAX_PSI streamfunction points (9,344 and 65,160) take the
    block-tridiagonal solve; the oracle solves with the reference's band LU.  psi, ub, u and u1
    within 1e-9 of each field's largest magnitude after three steps; the island integrals and
    corrections take the solve's unit-source responses from create."""
    from cgenie_gb300.goldstein import new_member_run
    mi, mj = shape
    m = grid.make_member(grid.MemberConfig(maxi=mi, maxj=mj, maxk=8, maxl=2, seed=62, mask="basin_island"))
    c = momentum.make_case(m, seed=9)
    assert c.maxi * (c.maxj + 1) > 8192 and c.isles >= 1
    g = new_member_run(m)
    mo = momentum.Momentum(c)
    mo.set_wind()
    o = ol.OracleMomentum(c)
    for _ in range(3):
        mo.step(g)
        o.step(m.rho)
    out, ref = mo.download(), o.state()
    for n in ("psi", "ub", "u", "u1"):
        close(out[n], ref[n], n)
    mo.close()
    g.close()


def test_ocean_step_momentum_then_tracers(gpu_lib):
    """Momentum then tstepo, four times, with density and velocities staying on the device."""
    from cgenie_gb300.goldstein import new_member_run
    m = grid.make_member(grid.MemberConfig(maxi=36, maxj=36, maxk=16, maxl=3, seed=55, mask="basin_island", diso=True))
    c = momentum.make_case(m, seed=6)
    g = new_member_run(m)
    mo = momentum.Momentum(c)
    mo.set_wind()
    o = ol.OracleMomentum(c)
    s = ol.OracleState(m)
    for _ in range(4):
        mo.step(g)
        g.tstepo(1)
        o.step(s.rho)
        s.u = np.ascontiguousarray(o.state()["u"])
        s.step(1)
    out = g.download()
    close(mo.download()["u"], o.state()["u"], "u")
    kk = np.arange(m.maxk + 2)[:, None, None]
    wet = (kk >= m.k1[None]) & (kk >= 1) & (kk <= m.maxk)
    wet[:, :, 0] = wet[:, :, -1] = False
    for l in range(m.maxl):
        close(out["ts"][..., l][wet], s.ts[..., l][wet], f"ts[{l}]")
    mo.close()
    g.close()


def test_errors(gpu_lib):
    from cgenie_gb300.goldstein import GoldsteinError, new_member_run
    m = grid.make_member(grid.MemberConfig(maxi=18, maxj=14, maxk=8, maxl=2, seed=56, mask="basin"))
    c = momentum.make_case(m, seed=7)
    mo = momentum.Momentum(c)
    g = new_member_run(m)
    with pytest.raises(GoldsteinError) as e:
        mo.step(g)                                   # before set_wind
    assert e.value.code == abi.GB_GO_ENOTREADY
    mo.set_wind()
    other = grid.make_member(grid.MemberConfig(maxi=20, maxj=14, maxk=8, maxl=2, seed=57, mask="basin"))
    g2 = new_member_run(other)
    with pytest.raises(GoldsteinError) as e:
        mo.step(g2)
    assert e.value.code == abi.GB_GO_EINVAL
    c.arrays["jpisl"] = c.arrays["jpisl"].copy()
    c.arrays["jpisl"][0, 0] = m.maxj                 # a path point on the last row
    with pytest.raises(GoldsteinError) as e:
        momentum.Momentum(c)
    assert e.value.code == abi.GB_GO_EINVAL
    for h in (g, g2):
        h.close()
    mo.close()


def test_split_precision_ocean_step(gpu_lib):
    """Momentum then tstepo on the split-precision form: the density is formed from its
    group-planar state and the transfer coefficients are rebuilt on the device from the new
    velocities.  u within 1e-9 of the oracle (FP64 tracer path), T and S within the form's
    bar for them (1e-11), the other tracers within 1e-6."""
    from cgenie_gb300.goldstein import new_member_run
    m = grid.make_member(grid.MemberConfig(maxi=36, maxj=36, maxk=16, maxl=4, seed=58, mask="basin_island",
                                           tracer_kind="bgc"))
    c = momentum.make_case(m, seed=8)
    g = new_member_run(m, precision=abi.GB_GO_FP32FLUX)
    mo = momentum.Momentum(c)
    mo.set_wind()
    o = ol.OracleMomentum(c)
    s = ol.OracleState(m)
    for _ in range(4):
        mo.step(g)
        g.tstepo(1)
        o.step(s.rho)
        s.u = np.ascontiguousarray(o.state()["u"])
        s.step(1)
    close(mo.download()["u"], o.state()["u"], "u")
    out = g.download()
    kk = np.arange(m.maxk + 2)[:, None, None]
    wet = (kk >= m.k1[None]) & (kk >= 1) & (kk <= m.maxk)
    wet[:, :, 0] = wet[:, :, -1] = False
    for l in range(m.maxl):
        a, b = out["ts"][..., l][wet], s.ts[..., l][wet]
        err = np.abs(a - b).max() / np.abs(b).max()
        assert err <= (1e-11 if l < 2 else 1e-6), (l, err)
    mo.close()
    g.close()
