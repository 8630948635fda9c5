"""Convective adjustment decisions on crafted columns, both precisions, bit-exact.

With zero velocities, zero diffusivities and no forcing a step leaves every tracer
value unchanged, so the adjustment (goldstein.f90:2657-2777) sees exactly the uploaded
columns.  The columns are built to reach every decision path of the batched
adjustment kernel: exact ties (bit-equal T and S), densities one ulp apart,
densities equal to rounding with different T and S, differences of ~1e-13,
strongly unstable and stable profiles.  The state after one step and the
convection counts (cost, including initial values where one addition per filled
level rounds differently from one addition of the count) must equal the oracle's
bit for bit."""
import numpy as np
import pytest

from cgenie_gb300 import abi, grid

pytestmark = pytest.mark.gpu


def crafted_member(seed, ieos=0, maxk=12, maxl=4):
    cfg = grid.MemberConfig(maxi=18, maxj=14, maxk=maxk, maxl=maxl, seed=seed, umax=0.0,
                            diff_h=1e-200, diff_v=1e-200, ieos=ieos, noise=0.0)
    m = grid.make_member(cfg)
    rng = np.random.default_rng(seed)
    ec = m.ec
    ts = m.ts
    for j in range(1, m.maxj + 1):
        for i in range(1, m.maxi + 1):
            k1 = int(m.k1[j, i])
            if k1 > m.maxk:
                continue
            lev = np.arange(k1, m.maxk + 1)
            n = len(lev)
            kind = (i + 2 * j) % 7
            t0 = rng.uniform(2.0, 20.0)
            s0 = rng.uniform(-1.0, 1.0)
            if kind == 0:      # stable: warmer upwards
                t = t0 + np.sort(rng.uniform(0.0, 5.0, n))
                s = np.full(n, s0)
            elif kind == 1:    # exact ties everywhere
                t = np.full(n, t0)
                s = np.full(n, s0)
            elif kind == 2:    # T one ulp apart, alternating
                t = np.where(np.arange(n) % 2 == 0, t0, np.nextafter(t0, np.inf))
                s = np.full(n, s0)
            elif kind == 3:    # random, mostly unstable
                t = rng.uniform(0.0, 25.0, n)
                s = rng.uniform(-2.0, 2.0, n)
            elif kind == 4:    # different T and S, densities equal to rounding
                t = rng.uniform(0.0, 25.0, n)
                r0 = ec[0] * t0 + ec[1] * s0 + ec[2] * (t0 * t0) + ec[3] * ((t0 * t0) * t0)
                s = (r0 - ec[0] * t - ec[2] * (t * t) - ec[3] * ((t * t) * t)) / ec[1]
            elif kind == 5:    # stable column with a cold surface level
                t = t0 + np.sort(rng.uniform(0.0, 5.0, n))
                t[-1] = t0 - 3.0
                s = np.full(n, s0)
            else:              # near ties ~1e-13 relative
                t = t0 * (1.0 + 1e-13 * rng.standard_normal(n))
                s = s0 * (1.0 + 1e-13 * rng.standard_normal(n))
            ts[lev, j, i, 0] = t
            ts[lev, j, i, 1] = s
            for l in range(2, m.maxl):
                ts[lev, j, i, l] = rng.uniform(0.5, 2.0, n)
    m.ts1[...] = ts
    m.rho[1:, :, :] = grid.eos_np(ec, ts[1:m.maxk + 1, :, :, 0], ts[1:m.maxk + 1, :, :, 1],
                                  m.zro[:, None, None], ieos)
    m.rho[0, 1:m.maxj + 1, 1:m.maxi + 1] = 0.0
    # convection counts: integers, non-integers (one addition per level differs from one
    # addition of the count) and a value where adding 1 rounds back
    c = rng.integers(0, 50, m.cost.shape).astype(np.float64)
    c[::3, ::2] += 0.1
    c[1, 1] = 2.0 ** 53
    m.cost[...] = c
    return m


def run_and_compare(oracle, m, precision):
    from cgenie_gb300.goldstein import new_member_run
    ref = oracle.OracleState(m)
    ref.step(1)
    g = new_member_run(m, precision=precision)
    g.tstepo(1)
    out = g.download()
    g.close()
    kk = np.arange(m.maxk + 2)[:, None, None]
    wet = (kk >= m.k1[None]) & (kk >= 1) & (kk <= m.maxk)
    wet[:, 0, :] = wet[:, -1, :] = False
    wet[:, :, 0] = wet[:, :, -1] = False
    for l in range(m.maxl):
        a = out["ts"][..., l][wet]
        b = ref.ts[..., l][wet]
        assert np.array_equal(a.view(np.int64), b.view(np.int64)), (l, int(np.sum(a != b)))
    assert np.array_equal(out["cost"].view(np.int64), ref.cost.view(np.int64))
    # the crafted columns do convect
    assert np.sum(ref.cost != m.cost) > 20


@pytest.mark.parametrize("precision", [abi.GB_GO_FP32FLUX, abi.GB_GO_FP64], ids=["fp32flux", "fp64"])
@pytest.mark.parametrize("seed,ieos", [(81, 0), (82, 0), (83, 1)], ids=["a", "b", "ieos1"])
def test_co_decisions_bit_exact(gpu_lib, oracle, precision, seed, ieos):
    run_and_compare(oracle, crafted_member(seed, ieos), precision)


# The split-precision form's two-phase adjustment at its limits: 32 levels (the longest
# merge logs: a column of exact ties merges 31 levels at once, a random one makes many
# merges), 24 and 32 tracers (30 replay slots per column over four tracer groups), and
# 3 tracers (one slot).
@pytest.mark.parametrize("precision", [abi.GB_GO_FP32FLUX, abi.GB_GO_FP64], ids=["fp32flux", "fp64"])
@pytest.mark.parametrize("seed,maxk,maxl", [(84, 32, 24), (85, 32, 32), (86, 16, 3)], ids=["k32l24", "k32l32", "k16l3"])
def test_co_decisions_deep_columns_bit_exact(gpu_lib, oracle, precision, seed, maxk, maxl):
    run_and_compare(oracle, crafted_member(seed, 0, maxk=maxk, maxl=maxl), precision)
