"""GPU checks of the restart writer (include/gb_restart.h): the file of a device-resident ocean
holds outm_netcdf's fields (src/goldstein/goldstein_data.f90:194-213) of the handle's current
state, bit for bit: against the oracle's steps for the FP64 form, against the handle's own
download for the split-precision form."""
import numpy as np
import pytest

from cgenie_gb300 import abi, grid
from oracle import oracle_lib as ol
from oracle import restart_np as orc

pytestmark = pytest.mark.gpu


def bits(a):
    return np.ascontiguousarray(a, dtype=np.float64).view(np.uint64)


def coords(m):
    return (np.linspace(0.0, 360.0, m.maxi, endpoint=False) + 5.0, np.linspace(-85.0, 85.0, m.maxj),
            np.cumsum(np.linspace(20.0, 600.0, m.maxk)))


def check_file(rs, path, m, ts, cal, gui=False, fluxes=None):
    from scipy.io import netcdf_file
    lon, lat, ncdepth = coords(m)
    want = orc.restart_fields(ts, m.u, m.k1, m.maxi, m.maxj, m.maxk)
    c, out = rs.read_goldstein(path, m.maxi, m.maxj, m.maxk, gui=gui)
    for n, w in zip(("temp", "salinity", "uvel", "vvel"), want):
        assert np.array_equal(bits(out[n]), bits(w)), n
    for n, f in zip(("evap", "late", "sens"), fluxes or (None,) * 3):
        assert np.array_equal(out[n], np.zeros((m.maxj, m.maxi)) if f is None else f), n
    assert (c.iyear, c.imonth, c.ioffset, c.day) == (cal.iyear, cal.imonth, cal.ioffset, float(orc.nint(cal.day)))
    with netcdf_file(path, "r", mmap=False) as nc:
        assert np.array_equal(nc.variables["depth"][:], orc.depths1(ncdepth))
        assert np.array_equal(bits(nc.variables["temp"][:]), bits(want[0]))


@pytest.mark.parametrize("steps", [0, 5])
def test_fp64_restart_matches_oracle(gpu_lib, tmp_path, steps):
    pytest.importorskip("scipy.io")
    from cgenie_gb300 import restart as rs
    from cgenie_gb300.goldstein import new_member_run
    m = grid.make_member(grid.MemberConfig(maxi=36, maxj=36, maxk=16, maxl=4, seed=61, mask="basin", diso=True))
    g = new_member_run(m)
    if steps:
        g.tstepo(steps)
    s = ol.OracleState(m)
    if steps:
        s.step(steps)
    cal = rs.Calendar(iyear=2000, imonth=3, ioffset=12, day=14.5)
    lon, lat, ncdepth = coords(m)
    r = np.random.default_rng(2)
    fl = [r.standard_normal((m.maxj, m.maxi)) for _ in range(3)]
    p = str(tmp_path / rs.goldstein_name(".", cal).split("/")[-1])
    rs.write_goldstein(g, p, cal, lon, lat, ncdepth, *fl)
    check_file(rs, p, m, s.ts, cal, fluxes=fl)
    # the handle keeps stepping after a write, as after outm_netcdf
    g.tstepo(2)
    s.step(2)
    assert np.array_equal(g.download()["ts"], s.ts)
    g.close()


def test_split_precision_restart_is_the_handle_state(gpu_lib, tmp_path):
    pytest.importorskip("scipy.io")
    from cgenie_gb300 import restart as rs
    from cgenie_gb300.goldstein import new_member_run
    m = grid.make_member(grid.MemberConfig(maxi=36, maxj=36, maxk=16, maxl=6, seed=62, mask="basin"))
    g = new_member_run(m, precision=abi.GB_GO_FP32FLUX)
    g.tstepo(4)
    cal = rs.Calendar(iyear=7, imonth=12, ioffset=0, day=30.7, istep=4)
    lon, lat, ncdepth = coords(m)
    p = str(tmp_path / "gui_restart_goldstein.nc")
    rs.write_goldstein(g, p, cal, lon, lat, ncdepth, gui=True)
    ts = g.download()["ts"]
    check_file(rs, p, m, ts, cal, gui=True)
    g.close()


def test_write_before_upload_is_refused(gpu_lib, tmp_path):
    from cgenie_gb300 import restart as rs
    from cgenie_gb300.goldstein import Goldstein, GoldsteinError
    m = grid.make_member(grid.MemberConfig(maxi=12, maxj=10, maxk=8, maxl=2, seed=63, mask="basin"))
    g = Goldstein(m)
    lon, lat, ncdepth = coords(m)
    with pytest.raises(GoldsteinError) as e:
        rs.write_goldstein(g, str(tmp_path / "x.nc"), rs.Calendar(), lon, lat, ncdepth)
    assert e.value.code == abi.GB_GO_ENOTREADY
    g.close()


def test_pack_is_the_file_data_section(gpu_lib):
    """gb_rs_pack_goldstein leaves in device memory the bytes the file holds for the four 3-D
    variables: big-endian doubles of outm_netcdf's fields."""
    import torch
    from cgenie_gb300 import restart as rs
    from cgenie_gb300.goldstein import new_member_run
    m = grid.make_member(grid.MemberConfig(maxi=36, maxj=36, maxk=16, maxl=3, seed=64, mask="basin"))
    g = new_member_run(m)
    g.tstepo(3)
    n = m.maxi * m.maxj * m.maxk
    dev = torch.full((4 * n,), float("nan"), dtype=torch.float64, device="cuda:0")
    rs.pack_goldstein(g, dev.data_ptr())
    torch.cuda.synchronize()
    got = dev.cpu().numpy().view(">f8").reshape(4, m.maxk, m.maxj, m.maxi)
    want = orc.restart_fields(g.download()["ts"], m.u, m.k1, m.maxi, m.maxj, m.maxk)
    for q in range(4):
        assert np.array_equal(bits(got[q]), bits(want[q])), q
    g.close()
