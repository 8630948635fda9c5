"""CPU checks of the GOLDSTEIN restart files (include/gb_restart.h, goldstein_data.f90:10-354).

The codec, the reader, the file name and the calendar are host code of the library and run
here without a GPU.  The encoding is pinned to the bytes of a file written by the netCDF
library (tests/golden/restart/main_restart_0.nc, the reference's own CDF-1 file of the same
scalar variables) and read back by an independent reader (scipy.io.netcdf_file); the calendar
and the file name against the oracle's restatement."""
import os

import numpy as np
import pytest

from cgenie_gb300 import abi
from oracle import restart_np as orc

GOLDEN = os.path.join(os.path.dirname(__file__), "golden", "restart", "main_restart_0.nc")


@pytest.fixture(scope="module")
def rs():
    from cgenie_gb300 import build
    build.build()
    from cgenie_gb300 import restart
    return restart


def bits(a):
    return np.ascontiguousarray(a, dtype=np.float64).view(np.uint64)


def case(seed=3, maxi=7, maxj=5, maxk=4):
    r = np.random.default_rng(seed)
    f = dict(lon=np.linspace(0.0, 350.0, maxi) + 5.0, lat=np.linspace(-80.0, 80.0, maxj),
             depths1=np.cumsum(r.uniform(10, 500, maxk))[::-1].copy())
    for n in ("temp", "salinity", "uvel", "vvel"):
        f[n] = r.standard_normal((maxk, maxj, maxi)) * 10.0
    f["temp"][:, 0, 1] = -0.0
    for n in ("evap", "late", "sens"):
        f[n] = r.standard_normal((maxj, maxi))
    return f


def write(rs, path, f, cal, gui=False):
    rs.write_fields(path, cal, f["lon"], f["lat"], f["depths1"], f["temp"], f["salinity"], f["uvel"], f["vvel"],
                    f["evap"], f["late"], f["sens"], gui=gui)


def var_entries(data: bytes):
    """name -> (header entry bytes without `begin`, begin) of a CDF-1 file (a minimal walk)."""
    be = lambda o: int.from_bytes(data[o:o + 4], "big")
    pad = lambda n: (n + 3) & ~3
    o = 8
    tag, n = be(o), be(o + 4)
    o += 8
    for _ in range(n):
        o += 4 + pad(be(o)) + 4
    o += 8   # no global attributes in these files
    tag, n = be(o), be(o + 4)
    assert tag == 0x0B
    o += 8
    out = {}
    for _ in range(n):
        start = o
        ln = be(o)
        name = data[o + 4:o + 4 + ln].decode()
        o += 4 + pad(ln)
        nd = be(o)
        o += 4 + 4 * nd
        atag, na = be(o), be(o + 4)
        o += 8
        for _ in range(na):
            o += 4 + pad(be(o))
            t, ne = be(o), be(o + 4)
            o += 8 + pad(ne * {1: 1, 2: 1, 3: 2, 4: 4, 5: 4, 6: 8}[t])
        o += 8
        out[name] = (data[start:o], be(o))
        o += 4
    return out


def test_golden_file_read_by_oracle_reader_and_library(rs):
    scipy_io = pytest.importorskip("scipy.io")
    with scipy_io.netcdf_file(GOLDEN, "r", mmap=False) as f:
        assert f.version_byte == 1
        vals = {k: int(f.variables[k][0]) for k in ("ioffset", "iyear", "imonth", "iday")}
    assert vals == dict(ioffset=0, iyear=2000, imonth=1, iday=2)
    cal, out = rs.read_goldstein(GOLDEN, 1, 1, 1, fields=())
    assert (cal.ioffset, cal.iyear, cal.imonth, cal.day) == (0, 2000, 1, 2.0)
    assert out == {}


def test_encoding_matches_netcdf_library_bytes(rs, tmp_path):
    gold = open(GOLDEN, "rb").read()
    p = str(tmp_path / "r.nc")
    cal = rs.Calendar(iyear=2000, imonth=1, ioffset=0, day=2.0)
    write(rs, p, case(), cal)
    mine = open(p, "rb").read()
    assert mine[:8] == gold[:8]                       # magic CDF-1, numrecs 0
    assert mine[8:16] == gold[8:16][:4] + (4).to_bytes(4, "big")   # dimension tag, 4 dimensions
    assert mine[16:32] == gold[16:32]                 # nrecs = 1, the first dimension
    ge, me = var_entries(gold), var_entries(mine)
    for name in ("ioffset", "iyear", "imonth", "iday"):
        assert me[name][0] == ge[name][0], name      # name, dims, attributes, type, vsize
        assert mine[me[name][1]:me[name][1] + 4] == gold[ge[name][1]:ge[name][1] + 4], name
    # data placement as the library's: first variable right after the header, then vsize apart
    begins = [b for _, b in ge.values()]
    assert begins[0] == len(gold) - 16 and np.all(np.diff(begins) == 4)
    mb = [b for _, b in me.values()]
    assert mb == sorted(mb)


@pytest.mark.parametrize("gui", [False, True])
def test_written_file_read_by_independent_reader(rs, tmp_path, gui):
    scipy_io = pytest.importorskip("scipy.io")
    f = case(seed=5)
    cal = rs.Calendar(iyear=1712, imonth=11, ioffset=37, day=17.4999, istep=123456)
    p = str(tmp_path / "g.nc")
    write(rs, p, f, cal, gui=gui)
    with scipy_io.netcdf_file(p, "r", mmap=False) as nc:
        assert nc.version_byte == 1
        assert dict(nc.dimensions) == dict(nrecs=1, longitude=7, latitude=5, depth=4)
        v = nc.variables
        names = ["longitude", "latitude", "depth", "ioffset", "iyear", "imonth", "iday"] + \
            (["istep_ocn"] if gui else []) + ["temp", "salinity", "uvel", "vvel", "evap", "late", "sens"]
        assert list(v) == names
        assert v["longitude"]._attributes == {"units": b"degrees_east", "long_name": b"longitude"}
        assert v["latitude"]._attributes == {"units": b"degrees_north", "long_name": b"latitude"}
        for n, ax in (("longitude", "lon"), ("latitude", "lat"), ("depth", "depths1")):
            assert v[n].typecode() == "f" and np.array_equal(v[n][:], f[ax].astype(np.float32))
        for n in ("temp", "salinity", "uvel", "vvel"):
            assert v[n].typecode() == "d" and v[n].dimensions == ("depth", "latitude", "longitude")
            assert np.array_equal(bits(v[n][:]), bits(f[n])), n   # incl. -0.0
        for n in ("evap", "late", "sens"):
            assert v[n].dimensions == ("latitude", "longitude") and np.array_equal(v[n][:], f[n])
        assert int(v["iday"][0]) == orc.nint(17.4999) == 17
        assert (int(v["iyear"][0]), int(v["imonth"][0]), int(v["ioffset"][0])) == (1712, 11, 37)
        if gui:
            assert int(v["istep_ocn"][0]) == 123456


def test_round_trip_through_the_library_reader(rs, tmp_path):
    f = case(seed=9, maxi=36, maxj=36, maxk=16)
    p = str(tmp_path / "rt.nc")
    write(rs, p, f, rs.Calendar(iyear=3, imonth=2, ioffset=5, day=29.5, istep=7), gui=True)
    cal, out = rs.read_goldstein(p, 36, 36, 16, gui=True)
    assert (cal.iyear, cal.imonth, cal.ioffset, cal.day, cal.istep) == (3, 2, 5, 30.0, 7)
    for n, a in out.items():
        assert np.array_equal(bits(a), bits(f[n])), n


def test_reader_converts_types_and_reads_cdf2(rs, tmp_path):
    scipy_io = pytest.importorskip("scipy.io")
    r = np.random.default_rng(1)
    p = str(tmp_path / "t.nc")
    with scipy_io.netcdf_file(p, "w", version=2) as nc:
        nc.createDimension("nrecs", 1)
        nc.createDimension("longitude", 3)
        nc.createDimension("latitude", 2)
        nc.createDimension("depth", 2)
        for n, t in (("ioffset", "i"), ("iyear", "h"), ("imonth", "b"), ("iday", "d")):
            nc.createVariable(n, t, ("nrecs",))[:] = {"ioffset": -4, "iyear": 300, "imonth": 12, "iday": 30.9}[n]
        t32 = r.standard_normal((2, 2, 3)).astype(np.float32)
        nc.createVariable("temp", "f", ("depth", "latitude", "longitude"))[:] = t32
        s16 = r.integers(-300, 300, (2, 2, 3)).astype(np.int16)
        nc.createVariable("salinity", "h", ("depth", "latitude", "longitude"))[:] = s16
    cal, out = rs.read_goldstein(p, 3, 2, 2, fields=("temp", "salinity"))
    assert (cal.ioffset, cal.iyear, cal.imonth, cal.day) == (-4, 300, 12, 30.0)   # 30.9 truncates
    assert np.array_equal(out["temp"], t32.astype(np.float64))
    assert np.array_equal(out["salinity"], s16.astype(np.float64))


def test_reader_errors(rs, tmp_path):
    from cgenie_gb300.goldstein import GoldsteinError
    f = case()
    p = str(tmp_path / "e.nc")
    write(rs, p, f, rs.Calendar())
    with pytest.raises(GoldsteinError, match="another shape"):
        rs.read_goldstein(p, 7, 5, 5)
    with pytest.raises(GoldsteinError, match="missing"):
        rs.read_goldstein(p, 7, 5, 4, gui=True)        # no istep_ocn in a plain restart
    with pytest.raises(GoldsteinError, match="missing file"):
        rs.read_goldstein(str(tmp_path / "none.nc"), 7, 5, 4)
    data = open(p, "rb").read()
    cut = str(tmp_path / "cut.nc")
    open(cut, "wb").write(data[:len(data) - 8])
    with pytest.raises(GoldsteinError, match="beyond the end"):
        rs.read_goldstein(cut, 7, 5, 4)
    h5 = str(tmp_path / "h5.nc")
    open(h5, "wb").write(b"\x89HDF\r\n\x1a\n" + bytes(64))
    with pytest.raises(GoldsteinError) as e:
        rs.read_goldstein(h5, 7, 5, 4)
    assert e.value.code == abi.GB_GO_EUNSUPPORTED


def test_grid_beyond_classic_format_refused(rs, tmp_path):
    """A 3-D variable that is not the file's last may not exceed 4 GiB - 4 bytes in the
    classic format (the netCDF library's NC_EVARSIZE): 536,870,912 cells are refused before
    any field is touched, 536,870,911 pass the size check."""
    from cgenie_gb300.goldstein import GoldsteinError
    p = str(tmp_path / "none.nc")
    with pytest.raises(GoldsteinError, match="classic format") as e:
        rs.read_goldstein(p, 1024, 1024, 512 + 1, fields=())
    assert e.value.code == abi.GB_GO_EINVAL
    with pytest.raises(GoldsteinError, match="classic format"):
        rs.read_goldstein(p, 7, 76695845, 1, fields=())   # 536,870,915 cells
    with pytest.raises(GoldsteinError, match="missing file"):
        rs.read_goldstein(p, 1, 536870911, 1, fields=())


def test_file_name_matches_oracle(rs):
    for y, m, d in [(0, 1, 1.0), (2000, 12, 30.5), (-5, 3, 2.49), (12345, 100, 14.6), (7, 7, 99.4), (7, 7, 99.6),
                    (-2147483647, 1, 1.0)]:
        cal = rs.Calendar(iyear=y, imonth=m, day=d)
        assert rs.goldstein_name("out/dir", cal) == orc.goldstein_name("out/dir", y, m, d), (y, m, d)
    assert rs.goldstein_name("o", rs.Calendar(iyear=2000, imonth=1, day=2.0)) == "o/goldstein_restart_2000_01_02.nc"


@pytest.mark.parametrize("yearlen,nyear", [(360.0, 100), (365.25, 96), (360.0, 48), (365.0, 7), (360.0, 360000)])
def test_calendar_matches_oracle(rs, yearlen, nyear):
    cal = rs.Calendar(iyear=1, imonth=1, day=1.0)
    y, m, d = 1, 1, 1.0
    for step in range(3 * nyear if nyear < 1000 else 2000):
        cal = rs.calendar_step(cal, yearlen, nyear)
        y, m, d = orc.calendar_step(y, m, d, yearlen, nyear)
        assert (cal.iyear, cal.imonth) == (y, m) and cal.day == d, step
    for ioff, iday in [(0, 1), (400, 30), (-400, 12), (1234567, 29)]:
        c = rs.calendar_after_read(rs.Calendar(iyear=5, imonth=12, ioffset=ioff, day=float(iday)), yearlen, nyear)
        assert (c.iyear, c.imonth, c.ioffset, c.day) == orc.calendar_after_read(5, 12, ioff, iday, yearlen, nyear)
