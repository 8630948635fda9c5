"""GPU checks of the split-precision form (FP32 transfers, FP64 state) and of the
batched ensemble.

Bars, per tracer, over wet cells, error = max|x - x_oracle| / max|x_oracle|:
  * T and S (double-float transfers):            <= 1e-11
  * every tracer, after 1000 steps:              <= 1e-6   (the stated FP32-flux bar)
  * convection counts (cost) equal to the oracle's
  * conservation of the compensated inventory sum(ts*ds*dz), zero forcing:
    drift <= 1e-12 relative
  * the kernel equals the CPU emulation of the same scheme (tests/fp32_emul.py)
    to 1e-13 (tracers other than T, S) -- a spec check of the kernel itself."""
import dataclasses

import numpy as np
import pytest

from cgenie_gb300 import abi, grid

pytestmark = pytest.mark.gpu

TOL_TS = 1e-11
TOL_REL = 1e-6
TOL_CONS = 1e-12


def wet_mask(m):
    kk = np.arange(m.maxk + 2)[:, None, None]
    w = (kk >= m.k1[None]) & (kk >= 1) & (kk <= m.maxk)
    w[:, 0, :] = False
    w[:, -1, :] = False
    w[:, :, 0] = False
    w[:, :, -1] = False
    return w


def tracer_errors(m, ts, ref):
    w = wet_mask(m)
    out = []
    for l in range(m.maxl):
        a = ts[..., l][w]
        b = ref[..., l][w]
        out.append(float(np.max(np.abs(a - b)) / max(np.max(np.abs(b)), 1e-300)))
    return np.array(out)


def run_fp32(m, steps):
    from cgenie_gb300.goldstein import new_member_run
    g = new_member_run(m, precision=abi.GB_GO_FP32FLUX)
    inv0 = g.inventory()
    g.tstepo(steps)
    out = g.download()
    out["inv0"] = inv0
    out["inv1"] = g.inventory()
    g.close()
    return out


def check_against_oracle(oracle, m, steps, tol_ts=TOL_TS, tol=TOL_REL):
    ref = oracle.OracleState(m)
    ref.step(steps)
    out = run_fp32(m, steps)
    err = tracer_errors(m, out["ts"], ref.ts)
    assert np.all(err[:2] <= tol_ts), ("T/S", err[:2])
    assert np.all(err <= tol), err
    assert np.array_equal(out["cost"], ref.cost), "convection counts differ"
    rel = np.abs(out["inv1"] - out["inv0"]) / np.abs(out["inv0"])
    assert np.all(rel <= TOL_CONS), rel
    return err


@pytest.mark.parametrize("cfg,steps", [
    (grid.config_c1(), 100),
    (grid.MemberConfig(maxi=36, maxj=36, maxk=16, maxl=9, seed=3, tracer_kind="bgc"), 100),
    (grid.MemberConfig(maxi=37, maxj=23, maxk=13, maxl=5, seed=51), 50),
    (grid.MemberConfig(maxi=18, maxj=18, maxk=32, maxl=24, seed=52, tracer_kind="bgc"), 50),
    # more than 32 levels: the adjustment's serial form
    (grid.MemberConfig(maxi=16, maxj=12, maxk=40, maxl=4, seed=57, noise=2.0), 30),
    # the split-precision limits: 64 levels, 32 tracers
    (grid.MemberConfig(maxi=10, maxj=8, maxk=64, maxl=32, seed=58, tracer_kind="bgc", noise=1.0), 10),
], ids=["c1", "l9", "odd", "deep24", "levels40", "max_k64_l32"])
def test_fp32_matches_oracle(gpu_lib, oracle, cfg, steps):
    check_against_oracle(oracle, grid.make_member(cfg), steps)


@pytest.mark.parametrize("cfg,steps", [
    (grid.config_c2(), 200),
    (grid.MemberConfig(maxi=37, maxj=23, maxk=13, maxl=5, seed=61, diso=True, slope_max=1e-3), 50),
], ids=["c2", "odd_diso"])
def test_fp32_isoneutral_matches_oracle(gpu_lib, oracle, cfg, steps):
    check_against_oracle(oracle, grid.make_member(cfg), steps, tol_ts=1e-9)


@pytest.mark.parametrize("cfg", [
    grid.MemberConfig(maxi=18, maxj=18, maxk=16, maxl=4, seed=91, iediff=1, ediffpow2=1.0, tracer_kind="bgc"),
    grid.MemberConfig(maxi=18, maxj=14, maxk=12, maxl=3, seed=92, iediff=2, ediffpow2=0.5, diso=True,
                      slope_max=1e-3),
    grid.MemberConfig(maxi=15, maxj=12, maxk=10, maxl=5, seed=93, iediff=1, ediffpow2=0.0, ieos=1, noise=1.0),
    grid.MemberConfig(maxi=15, maxj=12, maxk=10, maxl=3, seed=94, iediff=1, ediffpow2=0.7),
], ids=["pow1", "pow05_diso", "pow0_ieos", "pow07"])
def test_fp32_local_vertical_diffusivity(gpu_lib, oracle, cfg):
    """iediff 1/2 (goldstein.f90:2490-2516): the split-precision step rebuilds each cell's
    top-face coefficients from the step's FP64 T and S; within the FP32-flux bars."""
    check_against_oracle(oracle, grid.make_member(cfg), 40, tol_ts=1e-9)


def test_fp32_config2_1000_steps(gpu_lib, oracle):
    """Config 2 (36x36x16, 17 tracers, isoneutral) for its full 1000 steps."""
    err = check_against_oracle(oracle, grid.make_member(grid.config_c2()), 1000, tol_ts=1e-9)
    print("config 2, 1000 steps, per-tracer error:", " ".join(f"{e:.1e}" for e in err))


def test_fp32_kernel_equals_emulation(gpu_lib, oracle):
    from fp32_emul import Fp32Emulator
    from cgenie_gb300.goldstein import new_member_run
    for cfg in [grid.MemberConfig(maxi=36, maxj=36, maxk=16, maxl=9, seed=71, tracer_kind="bgc"),
                grid.MemberConfig(maxi=18, maxj=18, maxk=32, maxl=24, seed=72, tracer_kind="bgc")]:
        m = grid.make_member(cfg)
        em = Fp32Emulator(m, oracle)
        g = new_member_run(m, precision=abi.GB_GO_FP32FLUX)
        for _ in range(3):
            em.step(5)
            g.tstepo(5)
            out = g.download()
            err = tracer_errors(m, out["ts"], em.ts)
            assert np.all(err[2:] <= 1e-13), err
            assert np.all(err[:2] <= 1e-12), err
        g.close()


def test_fp32_offset_tracers_divergent_velocity(gpu_lib, oracle):
    """Tracers with an offset (DIC, alkalinity: T = tref + T', the FP32 transfers carry T')
    under a velocity field whose faces do not cancel (east velocities scaled, w kept): the
    offset's share tref * D enters per cell; within the bars of the oracle, and equal to the
    CPU emulation of the scheme to 1e-13."""
    import dataclasses
    from fp32_emul import Fp32Emulator, divergence_pair, coefficients, offsets
    from cgenie_gb300.goldstein import new_member_run
    m = grid.make_member(grid.MemberConfig(maxi=18, maxj=14, maxk=8, maxl=6, seed=95, tracer_kind="bgc"))
    u = m.u.copy()
    u[2:5, :, :, 0] *= 1.25
    m = dataclasses.replace(m, u=np.ascontiguousarray(u))
    assert np.any(offsets(m, m.ts) != 0)
    c32, lo, _ = coefficients(m)
    assert np.any(divergence_pair(m, c32, lo)[0] != 0)
    em = Fp32Emulator(m, oracle)
    g = new_member_run(m, precision=abi.GB_GO_FP32FLUX)
    em.step(6)
    g.tstepo(6)
    err = tracer_errors(m, g.download()["ts"], em.ts)
    assert np.all(err[2:] <= 1e-13), err
    g.tstepo(34)
    out = g.download()
    g.close()
    ref = oracle.OracleState(m)
    ref.step(40)
    err = tracer_errors(m, out["ts"], ref.ts)
    assert np.all(err[:2] <= TOL_TS), err
    assert np.all(err <= TOL_REL), err
    assert np.array_equal(out["cost"], ref.cost)


def test_fp32_forcing_and_branches(gpu_lib, oracle):
    for cfg in [grid.MemberConfig(maxi=18, maxj=14, maxk=8, maxl=3, seed=53, forcing=1.0),
                grid.MemberConfig(maxi=18, maxj=14, maxk=8, maxl=3, seed=54, iconv=1, ieos=1, diso=True, noise=2.0)]:
        m = grid.make_member(cfg)
        ref = oracle.OracleState(m)
        ref.step(20)
        out = run_fp32(m, 20)
        err = tracer_errors(m, out["ts"], ref.ts)
        assert np.all(err[:2] <= 1e-9), (cfg, err)
        assert np.all(err <= TOL_REL), (cfg, err)


def test_ensemble_alone_equals_in_mix(gpu_lib):
    """A member's result is the same (bit for bit) alone and in a mixed batch."""
    from cgenie_gb300.ensemble import Ensemble
    cfgs = grid.ensemble_configs(n=9, seed=9)
    mems = [grid.make_member(c) for c in cfgs]
    alone = Ensemble()
    aid = alone.add(mems[4])
    alone.step(30)
    a = alone.download(aid)
    alone.close()
    mix = Ensemble()
    ids = [mix.add(m) for m in mems]
    mix.step(30)
    b = mix.download(ids[4])
    assert np.array_equal(a["ts"], b["ts"])
    # staggered admission: a member admitted later runs the same 30 steps
    late = mix.add(mems[4], steps=30)
    mix.step(45)
    c = mix.download(late)
    assert np.array_equal(a["ts"], c["ts"])
    assert mix.remaining(late) == 0
    mix.close()


CO_FORMS = pytest.mark.parametrize("co_form", [abi.GB_ENS_CO_WARP, abi.GB_ENS_CO_TWO_PHASE], ids=["warp", "two_phase"])


@CO_FORMS
def test_ensemble_matches_oracle_per_member(gpu_lib, oracle, co_form):
    from cgenie_gb300.ensemble import Ensemble
    cfgs = grid.ensemble_configs(n=6, seed=11)
    mems = [grid.make_member(c) for c in cfgs]
    ens = Ensemble(use_graph=True, co_form=co_form)
    ids = [ens.add(m) for m in mems]
    inv0 = [ens.inventory(i) for i in ids]
    ens.step(20)
    ens.step(20)
    for m, i, v0 in zip(mems, ids, inv0):
        ref = oracle.OracleState(m)
        ref.step(40)
        out = ens.download(i)
        err = tracer_errors(m, out["ts"], ref.ts)
        assert np.all(err[:2] <= TOL_TS), err
        assert np.all(err <= TOL_REL), err
        assert np.array_equal(out["cost"], ref.cost)
        v1 = ens.inventory(i)
        assert np.all(np.abs(v1 - v0) <= TOL_CONS * np.abs(v0))
        assert ens.status(i) == 0
    ens.close()


@CO_FORMS
def test_ensemble_mixed_adjustment_forms(gpu_lib, oracle, co_form):
    """One batch with members of both adjustment paths: warp-parallel or two-phase (ieos = 0,
    iconv = 0, maxk <= 32) and serial (ieos = 1 with coshuffle; 40 levels), and a member
    with the local vertical diffusivity (iediff = 1)."""
    from cgenie_gb300.ensemble import Ensemble
    mems = [grid.make_member(grid.MemberConfig(maxi=18, maxj=14, maxk=16, maxl=5, seed=61, noise=2.0,
                                               tracer_kind="bgc")),
            grid.make_member(grid.MemberConfig(maxi=15, maxj=12, maxk=10, maxl=3, seed=62, ieos=1, iconv=1,
                                               noise=2.0)),
            grid.make_member(grid.MemberConfig(maxi=16, maxj=12, maxk=40, maxl=4, seed=63, noise=2.0)),
            grid.make_member(grid.MemberConfig(maxi=18, maxj=14, maxk=16, maxl=4, seed=64, iediff=1,
                                               ediffpow2=1.0, tracer_kind="bgc"))]
    ens = Ensemble(use_graph=True, co_form=co_form)
    ids = [ens.add(m) for m in mems]
    ens.step(25)
    for m, i in zip(mems, ids):
        ref = oracle.OracleState(m)
        ref.step(25)
        out = ens.download(i)
        err = tracer_errors(m, out["ts"], ref.ts)
        assert np.all(err[:2] <= TOL_TS), err
        assert np.all(err <= TOL_REL), err
        assert np.array_equal(out["cost"], ref.cost)
        assert ens.status(i) == 0
    ens.close()


def test_ensemble_budget_and_removal(gpu_lib):
    from cgenie_gb300.ensemble import Ensemble
    from cgenie_gb300.goldstein import GoldsteinError
    m = grid.make_member(grid.MemberConfig(maxi=18, maxj=18, maxk=16, maxl=4, seed=55))
    nb = Ensemble.member_bytes(m)
    ens = Ensemble(hbm_budget_bytes=int(2.5 * nb))
    a = ens.add(m)
    b = ens.add(m)
    with pytest.raises(GoldsteinError) as ex:
        ens.add(m)
    assert ex.value.code == abi.GB_GO_ENOMEM
    ens.remove(a)
    c = ens.add(m)
    ens.step(3)
    assert ens.count()[0] == 2
    ens.remove(b)
    ens.remove(c)
    ens.close()


def test_fp32_velocity_updates_on_device(gpu_lib, oracle):
    """A velocity field set after the first is turned into coefficients on the device:
    the same field gives the run bit for bit, a new field stays within the bars against
    the FP64 oracle run on that field."""
    from cgenie_gb300.goldstein import new_member_run
    m = grid.make_member(grid.MemberConfig(maxi=36, maxj=36, maxk=16, maxl=9, seed=91, tracer_kind="bgc"))
    g1 = new_member_run(m, precision=abi.GB_GO_FP32FLUX)
    g2 = new_member_run(m, precision=abi.GB_GO_FP32FLUX)
    g2.set_velocity()                    # second field: device path, same values
    g1.tstepo(20)
    g2.tstepo(20)
    a, b = g1.download(), g2.download()
    assert np.array_equal(a["ts"], b["ts"])
    u2 = m.u * 0.7
    g2.set_velocity(u2)
    g2.tstepo(30)
    out = g2.download()
    g1.close()
    g2.close()
    import dataclasses
    m2 = dataclasses.replace(m)
    m2.u = u2
    ref = oracle.OracleState(m)
    ref.step(20)
    ref.u = np.ascontiguousarray(u2)
    ref.step(30)
    err = tracer_errors(m, out["ts"], ref.ts)
    assert np.all(err[:2] <= 1e-9), err
    assert np.all(err <= TOL_REL), err


def test_ensemble_parallel_admission_equals_serial(gpu_lib):
    """Members admitted in one batched call (add_many: host preparation on several threads,
    device set-up batched) step to the same result, bit for bit, as members admitted one by
    one."""
    from cgenie_gb300.ensemble import Ensemble
    mems = [grid.make_member(c) for c in grid.ensemble_configs(n=12, seed=21)]
    a = Ensemble(use_graph=True)
    ids_a = [a.add(m) for m in mems]
    b = Ensemble(use_graph=True)
    ids_b = b.add_many(mems)
    assert len(set(ids_b)) == len(mems)
    a.step(15)
    b.step(15)
    for ia, ib in zip(ids_a, ids_b):
        oa, ob = a.download(ia), b.download(ib)
        assert np.array_equal(oa["ts"], ob["ts"])
        assert np.array_equal(oa["cost"], ob["cost"])
    a.close()
    b.close()


def test_ensemble_batched_download_equals_export_path(gpu_lib):
    """download_many (gb_ens_download_many: one kernel for all members, copies queued behind the
    steps, one synchronisation; into new or caller-given arrays) returns what the
    export-then-merge path of gb_ens_download_stream returns, bit for bit, for ts, rho and
    cost."""
    from cgenie_gb300.abi import dptr
    from cgenie_gb300.ensemble import Ensemble
    mems = [grid.make_member(c) for c in grid.ensemble_configs(n=9, seed=23)]
    mems.append(grid.make_member(grid.MemberConfig(maxi=15, maxj=12, maxk=10, maxl=3, seed=62, ieos=1, iconv=1,
                                                   noise=2.0)))
    e = Ensemble(use_graph=True)
    ids = e.add_many(mems)
    e.step(12)
    par = e.download_many(ids)
    given = [dict(ts=np.zeros_like(m.ts), rho=np.zeros_like(m.rho), cost=np.zeros_like(m.cost)) for m in mems]
    e.download_many(ids, out=given)
    for i, m, p, g in zip(ids, mems, par, given):
        s = dict(ts=np.empty_like(m.ts), rho=np.empty_like(m.rho), cost=np.empty_like(m.cost))
        rc = e.lib.gb_ens_download_stream(e.e, int(i), None, dptr(s["ts"]), dptr(s["rho"]), dptr(s["cost"]))
        assert rc == 0
        for k in ("ts", "rho", "cost"):
            assert np.array_equal(s[k], p[k]), k
            assert np.array_equal(s[k], g[k]), k
    e.close()


def test_ensemble_mapped_host_arrays(gpu_lib):
    """Arrays in mapped page-locked host memory (gb_ens_host_alloc): add_many reads ts and u
    through the device address in its scatter kernel and download_many writes ts, rho and cost
    there from its kernel.  Results equal those of ordinary host arrays bit for bit, every
    element of the outputs is written, and gb_ens_host_free refuses a pointer it did not
    allocate."""
    import ctypes as C
    import dataclasses
    from cgenie_gb300.ensemble import Ensemble, host_copy, host_empty
    mems = [grid.make_member(c) for c in grid.ensemble_configs(n=9, seed=27)]
    mems.append(grid.make_member(grid.MemberConfig(maxi=16, maxj=12, maxk=40, maxl=4, seed=63, noise=2.0)))
    hmems = [dataclasses.replace(m, ts=host_copy(m.ts), u=host_copy(m.u)) for m in mems]
    a = Ensemble(use_graph=True)
    ids_a = a.add_many(mems)
    b = Ensemble(use_graph=True)
    ids_b = b.add_many(hmems)
    a.step(11)
    b.step(11)
    ref = a.download_many(ids_a)
    outs = []
    for m in mems:
        o = dict(ts=host_empty(m.ts.shape), rho=host_empty(m.rho.shape), cost=host_empty(m.cost.shape))
        for v in o.values():
            v[...] = np.nan
        outs.append(o)
    b.download_many(ids_b, out=outs)
    for r, o in zip(ref, outs):
        for k in ("ts", "rho", "cost"):
            assert not np.isnan(o[k]).any(), k
            assert np.array_equal(r[k], o[k]), k
    junk = np.zeros(4)
    assert a.lib.gb_ens_host_free(C.c_void_p(junk.ctypes.data)) != 0
    a.close()
    b.close()


def test_ensemble_packing_and_cta_cap_do_not_change_results(gpu_lib):
    """The member packing (order of the work items) and the cap on resident CTAs per SM change
    only which CTA takes which item: every member's result is bit-identical, and a bad value is
    refused."""
    from cgenie_gb300 import abi
    from cgenie_gb300.ensemble import Ensemble
    from cgenie_gb300.goldstein import GoldsteinError
    mems = [grid.make_member(c) for c in grid.ensemble_configs(n=12, seed=29)]
    ref = None
    for packing, cap in ((abi.GB_ENS_PACK_MEMBERS, 0), (abi.GB_ENS_PACK_ITEMS, 0), (abi.GB_ENS_PACK_ROUND_ROBIN, 2),
                         (abi.GB_ENS_PACK_ITEMS, 1)):
        e = Ensemble(use_graph=True, packing=packing, ctas_per_sm=cap)
        ids = e.add_many(mems)
        e.step(9)
        out = e.download_many(ids)
        e.close()
        if ref is None:
            ref = out
            continue
        for a, b in zip(ref, out):
            for k in ("ts", "rho", "cost"):
                assert np.array_equal(a[k], b[k]), (packing, cap, k)
    e = Ensemble()
    with pytest.raises(GoldsteinError):
        e.set_tuning(packing=7)
    with pytest.raises(GoldsteinError):
        e.set_tuning(ctas_per_sm=-1)
    e.co_form = 3
    with pytest.raises(GoldsteinError):
        e.set_tuning()
    e.close()


def _with_mask(m, k1):
    """Member m with the interior mask k1 (maxj, maxi) and the periodic halo columns."""
    import dataclasses
    full = m.k1.copy()
    full[1:-1, 1:-1] = k1
    full[:, 0] = full[:, m.maxi]
    full[:, m.maxi + 1] = full[:, 1]
    return dataclasses.replace(m, k1=full)


def test_ensemble_degenerate_members(gpu_lib):
    """Edge cases in one batch: a member without any wet column, a member with one wet column,
    the smallest grid (2x2x2, T and S), and the largest member shape (64 levels, 32 tracers),
    next to an ordinary member.  Each equals its FP64 run within the split-precision bars (the
    land-only member exactly its upload), and the ordinary member equals its run in a batch of
    its own bit for bit."""
    from cgenie_gb300.ensemble import Ensemble
    from cgenie_gb300.goldstein import new_member_run
    from test_gpu_long import per_tracer_errors
    base = grid.make_member(grid.MemberConfig(maxi=12, maxj=10, maxk=8, maxl=5, seed=71, tracer_kind="bgc"))
    land = _with_mask(base, np.full((base.maxj, base.maxi), base.maxk + 1, dtype=np.int32))
    one = np.full((base.maxj, base.maxi), base.maxk + 1, dtype=np.int32)
    one[4, 5] = 1
    single = _with_mask(base, one)
    tiny = grid.make_member(grid.MemberConfig(maxi=2, maxj=2, maxk=2, maxl=2, seed=72))
    big = grid.make_member(grid.MemberConfig(maxi=10, maxj=8, maxk=64, maxl=32, seed=58, tracer_kind="bgc", noise=1.0))
    normal = grid.make_member(grid.MemberConfig(maxi=18, maxj=14, maxk=16, maxl=7, seed=73, tracer_kind="bgc"))
    mems = [land, single, tiny, big, normal]
    e = Ensemble(use_graph=True)
    ids = e.add_many(mems)
    e.step(12)
    outs = e.download_many(ids)
    solo = Ensemble(use_graph=True)
    sid = solo.add_many([normal])
    solo.step(12)
    assert np.array_equal(solo.download_many(sid)[0]["ts"], outs[4]["ts"])
    solo.close()
    assert np.array_equal(outs[0]["ts"], land.ts)
    for m, out, mid in zip(mems[1:], outs[1:], ids[1:]):
        g = new_member_run(m, precision=abi.GB_GO_FP64)
        g.tstepo(12)
        ref = g.download()
        g.close()
        if (m.k1[1:-1, 1:-1] <= m.maxk).any():
            err = per_tracer_errors(m, out["ts"], ref["ts"])
            assert np.all(err[:2] <= 1e-11) and np.all(err <= 1e-6), (m.maxi, m.maxk, m.maxl, err)
        assert np.array_equal(out["cost"], ref["cost"])
        assert e.status(mid) == 0
    e.close()


def test_ensemble_adjustment_scratch_grows(gpu_lib):
    """The two-phase adjustment's merge logs and tracer slots are sized by the batch (listable
    columns x (largest L - 2)); members with more tracers admitted later grow them.  Every
    member equals its run alone, bit for bit, before and after the growth."""
    from cgenie_gb300.ensemble import Ensemble
    small = [grid.make_member(grid.MemberConfig(maxi=18, maxj=18, maxk=16, maxl=2, seed=s, noise=2.0)) for s in (701, 702)]
    big = [grid.make_member(grid.MemberConfig(maxi=36, maxj=36, maxk=32, maxl=l, seed=s, noise=2.0, tracer_kind="bgc"))
           for s, l in ((703, 24), (704, 32))]

    def alone(m, steps):
        e = Ensemble(use_graph=True, co_form=abi.GB_ENS_CO_TWO_PHASE)
        i = e.add_many([m])
        e.step(steps)
        out = e.download_many(i)[0]["ts"]
        e.close()
        return out

    e = Ensemble(use_graph=True, co_form=abi.GB_ENS_CO_TWO_PHASE)
    ids = e.add_many(small)
    e.step(6)
    for i, m in zip(ids, small):
        assert np.array_equal(e.download_many([i])[0]["ts"], alone(m, 6))
    bid = e.add_many(big)
    e.step(6)
    for i, m in zip(ids, small):
        assert np.array_equal(e.download_many([i])[0]["ts"], alone(m, 12))
    for i, m in zip(bid, big):
        assert np.array_equal(e.download_many([i])[0]["ts"], alone(m, 6))
    assert all(e.status(i) == 0 for i in ids + bid)
    e.close()


def test_ensemble_adjustment_forms_agree(gpu_lib):
    """The one-warp-per-column and two-phase adjustments give the same state and convection
    counts bit for bit, on convecting members of every shape and tracer count (and both at
    once in the automatic form's choice for this small batch)."""
    from cgenie_gb300.ensemble import Ensemble
    cfgs = grid.ensemble_configs(n=9, seed=21)
    mems = [grid.make_member(dataclasses.replace(c, noise=2.0)) for c in cfgs]
    outs = {}
    for form in (abi.GB_ENS_CO_WARP, abi.GB_ENS_CO_TWO_PHASE, abi.GB_ENS_CO_AUTO):
        e = Ensemble(use_graph=True, co_form=form)
        ids = e.add_many(mems)
        e.step(30)
        outs[form] = [e.download(i) for i in ids]
        assert all(e.status(i) == 0 for i in ids)
        e.close()
    for a, b, c in zip(*outs.values()):
        for k in ("ts", "cost"):
            assert np.array_equal(a[k], b[k]) and np.array_equal(a[k], c[k]), k
    # the members do convect
    assert sum(int(np.sum(o["cost"] != m.cost)) for o, m in zip(outs[abi.GB_ENS_CO_WARP], mems)) > 100
