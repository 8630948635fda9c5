"""GOLDSTEIN time-series diagnostics (include/gb_timeseries.h): diag2 and diagopsi
(src/goldstein/goldstein_diag.f90:10-71, 350-411) on the device-resident state, and the
.t/.s/.opsit records of step_goldstein (goldstein.f90:284-310, formats 100 and 110).

* CPU: the records' E14.6 fields against known Fortran renderings; the oracle's diagnostics
  on known answers (a uniform tracer has that value as every regional mean; no flow gives
  zero streamfunctions and avs).
* GPU: every number equals the oracle's (oracle/timeseries_oracle.c, the reference's loop and
  operation order) bit for bit, for the FP64 form after steps (the state is the oracle's), for
  the split-precision form (against the oracle on the handle's own downloaded state), with a
  split Atlantic, and on the reference's real masks."""
import os

import numpy as np
import pytest

from cgenie_gb300 import abi, grid
from cgenie_gb300.timeseries import OPSISC, format_records, make_basins

MASKS = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden", "masks")

# Fortran E14.6 renderings (gfortran) of values, right-justified in 14 characters
KNOWN = [
    (1.0, "  0.100000E+01"), (-123.456, " -0.123456E+03"), (1e-5, "  0.100000E-04"),
    (0.0, "  0.000000E+00"), (2.5e-7, "  0.250000E-06"), (999999.5, "  0.100000E+07"),
    (1e120, "  0.100000+121"), (-3.0e-150, " -0.300000-149"), (0.1234564, "  0.123456E+00"),
    (0.1234566, "  0.123457E+00"), (6.02e23, "  0.602000E+24"),
]


def test_records_fortran_format(gpu_lib_host):
    vals = [v for v, _ in KNOWN]
    sums = np.array((vals * 2)[:16])
    t, s, o = format_records(vals[0], 2, sums, 1.5, -2.25, np.array([-1.0, 2.0, -3.0, 4.0]) / OPSISC,
                             np.array([12, 7], np.int32))
    fields = [t[14 * n:14 * (n + 1)] for n in range(11)]
    assert t.endswith("\n") and len(t) == 11 * 14 + 1
    assert fields[0] == KNOWN[0][1]
    assert fields[1:9] == [f for _, f in (KNOWN * 2)[:8]]
    assert fields[9] == "  0.150000E+01" and fields[10] == " -0.225000E+01"
    assert s[14:14 * 9] == "".join(f for _, f in (KNOWN * 2)[8:16])
    assert o == "  0.100000E+01 -0.100000E+01  0.200000E+01 -0.300000E+01  0.400000E+01   12    7\n"


@pytest.fixture(scope="module")
def gpu_lib_host():
    """The library for its host-only entry points (no GPU needed)."""
    from cgenie_gb300 import build
    build.build()
    from cgenie_gb300 import goldstein
    return goldstein.load_library()


def test_oracle_known_answers(oracle):
    m = grid.make_member(grid.MemberConfig(maxi=18, maxj=14, maxk=8, maxl=3, seed=3, umax=0.0))
    ts = m.ts.copy()
    ts[..., 2] = 7.25
    b = make_basins(m.maxi, m.maxj, m.maxk)
    r = oracle.timeseries(m, ts, m.rho, m.u, b)
    means = r["sums"][16:24]
    assert np.all(np.abs(means[means != 0] - 7.25) <= 1e-14 * 7.25)
    assert r["avs"] == 0.0
    assert np.all(r["opsi"] == 0) and np.all(r["opsia"] == 0) and np.all(r["ext"] == 0)


def _check_equal(out, ref, m):
    for k in ("sums", "ext", "iposa", "opsi", "opsip", "opsia"):
        assert np.array_equal(out[k], ref[k]), k
    assert out["avn"] == ref["avn"] and out["avs"] == ref["avs"]
    assert np.any(out["sums"] != 0) and out["avs"] > 0 and np.any(out["opsi"] != 0)


@pytest.mark.gpu
@pytest.mark.parametrize("kw,split", [
    (dict(maxi=36, maxj=36, maxk=16, maxl=6, seed=21, diso=True, slope_max=1e-3, tracer_kind="bgc"), False),
    (dict(maxi=37, maxj=23, maxk=13, maxl=3, seed=22), True),
    (dict(maxi=36, maxj=36, maxk=16, maxl=4, seed=23, mask="file", mask_file=os.path.join(MASKS, "worjh2")), False),
    (dict(maxi=36, maxj=36, maxk=8, maxl=2, seed=24, mask="file", mask_file=os.path.join(MASKS, "worbe2")), True),
], ids=["36x36x16_diso", "odd_split", "worjh2", "worbe2_split"])
def test_fp64_diagnostics_equal_oracle(gpu_lib, oracle, kw, split):
    from cgenie_gb300.goldstein import new_member_run
    from cgenie_gb300.timeseries import TimeSeries
    m = grid.make_member(grid.MemberConfig(**kw))
    b = make_basins(m.maxi, m.maxj, m.maxk, split_atlantic=split)
    g = new_member_run(m, precision=abi.GB_GO_FP64)
    tsd = TimeSeries(m, b)
    # before any step (the uploaded state), then after steps (the oracle's state bit for bit)
    _check_equal(tsd.diagnose(g, streamfunctions=True), oracle.timeseries(m, m.ts, m.rho, m.u, b), m)
    ref = oracle.OracleState(m)
    ref.step(15)
    g.tstepo(15)
    out = tsd.diagnose(g, streamfunctions=True)
    _check_equal(out, oracle.timeseries(m, ref.ts, ref.rho, m.u, b), m)
    t, s, o = TimeSeries.records(15 / 96.0, m.maxl, out)
    assert len(t.splitlines()[0]) == 154 and len(o.splitlines()[0]) == 80
    tsd.close()
    g.close()


@pytest.mark.gpu
def test_split_precision_diagnostics_on_its_state(gpu_lib, oracle):
    from cgenie_gb300.goldstein import new_member_run
    from cgenie_gb300.timeseries import TimeSeries
    m = grid.make_member(grid.MemberConfig(maxi=36, maxj=36, maxk=16, maxl=9, seed=25, tracer_kind="bgc"))
    b = make_basins(m.maxi, m.maxj, m.maxk)
    g = new_member_run(m, precision=abi.GB_GO_FP32FLUX)
    g.tstepo(12)
    tsd = TimeSeries(m, b)
    out = tsd.diagnose(g, streamfunctions=True)
    st = g.download()
    _check_equal(out, oracle.timeseries(m, st["ts"], st["rho"], m.u, b), m)
    tsd.close()
    g.close()


def test_bad_basins_refused(gpu_lib_host):
    from cgenie_gb300.goldstein import GoldsteinError
    from cgenie_gb300.timeseries import TimeSeries
    m = grid.make_member(grid.MemberConfig(maxi=12, maxj=10, maxk=6, maxl=2, seed=4))
    b = make_basins(m.maxi, m.maxj, m.maxk)
    b.ipf = b.ipf.copy()
    b.ipf[3] = m.maxi + 5
    with pytest.raises(GoldsteinError) as e:
        TimeSeries(m, b)
    assert e.value.code == abi.GB_GO_EINVAL
