"""GOLDSTEIN time-series diagnostics of a device-resident ocean (include/gb_timeseries.h):
diag2 and diagopsi (src/goldstein/goldstein_diag.f90:10-71, 350-411) on a :class:`Goldstein`
handle's state, and the .t/.s/.opsit records of step_goldstein (goldstein.f90:284-310).

:func:`make_basins` gives seeded basin rows (Pacific and Atlantic longitude ranges per
latitude row, the Southern Ocean rows) for synthetic grids; a model passes the rows
initialise_goldstein derives from its .bmask file.
"""
from __future__ import annotations

import ctypes as C
from dataclasses import dataclass

import numpy as np

from .abi import GridRefs, GbDims, GbGrid, dptr
from .goldstein import GoldsteinError, load_library

OPSISC = 5e3 * 0.05 * 6.37e6 * 1.0e-6   # dsc * usc * rsc * 1e-6 (goldstein_lib.f90:60)

_ip = C.POINTER(C.c_int32)


class GbTsBasins(C.Structure):
    _fields_ = [("ips", _ip), ("ipf", _ip), ("ias", _ip), ("iaf", _ip), ("jsf", C.c_int32), ("overdep", C.c_int32)]


@dataclass
class Basins:
    ips: np.ndarray    # (maxj,) int32, rows 1..maxj
    ipf: np.ndarray
    ias: np.ndarray
    iaf: np.ndarray
    jsf: int
    overdep: int

    def c(self):
        self._keep = [np.ascontiguousarray(a, dtype=np.int32) for a in (self.ips, self.ipf, self.ias, self.iaf)]
        return GbTsBasins(*[a.ctypes.data_as(_ip) for a in self._keep], int(self.jsf), int(self.overdep))


def make_basins(maxi: int, maxj: int, maxk: int, split_atlantic: bool = False) -> Basins:
    """Seeded-free basin rows: Pacific over the second sixth to the half of the longitudes,
    Atlantic over the last third (or, split, through i = maxi into the first columns), the
    Southern Ocean up to a fifth of the rows; overturning extrema over the lower three
    quarters of the levels."""
    ips = np.full(maxj, max(1, maxi // 6), np.int32)
    ipf = np.full(maxj, max(1, maxi // 2), np.int32)
    if split_atlantic:
        ias = np.full(maxj, min(maxi, (5 * maxi) // 6), np.int32)
        iaf = np.full(maxj, max(1, maxi // 12), np.int32)
    else:
        ias = np.full(maxj, min(maxi, (2 * maxi) // 3), np.int32)
        iaf = np.full(maxj, maxi, np.int32)
    return Basins(ips, ipf, ias, iaf, jsf=max(0, maxj // 5), overdep=max(1, (3 * maxk) // 4))


class TimeSeries:
    """The diagnostics of one grid (gb_ts handle); diagnose() reads a Goldstein handle."""

    def __init__(self, member, basins: Basins, device: int = -1):
        self.lib = load_library()
        self.m = member
        self.refs = GridRefs(member)
        self.basins = basins
        self._cb = basins.c()
        h = C.c_void_p()
        rc = self.lib.gb_ts_create(C.byref(self.refs.dims), C.byref(self.refs.grid), C.byref(self._cb), int(device),
                                   C.byref(h))
        if rc != 0:
            raise GoldsteinError(rc, "gb_ts_create")
        self.h = h

    def close(self):
        if getattr(self, "h", None):
            self.lib.gb_ts_destroy(self.h)
            self.h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def diagnose(self, ocean, streamfunctions: bool = False) -> dict:
        m = self.m
        sums = np.zeros(8 * m.maxl)
        avn, avs = C.c_double(), C.c_double()
        ext = np.zeros(4)
        iposa = np.zeros(2, np.int32)
        shape = (m.maxk + 1, m.maxj + 1)     # Fortran (0:maxj, 0:maxk)
        ops = [np.zeros(shape) for _ in range(3)] if streamfunctions else [None] * 3
        rc = self.lib.gb_ts_diagnose(self.h, ocean.h, dptr(sums), C.byref(avn), C.byref(avs), dptr(ext),
                                     iposa.ctypes.data_as(_ip), *[dptr(a) for a in ops])
        if rc != 0:
            raise GoldsteinError(rc, "gb_ts_diagnose", self.lib.gb_ts_last_error(self.h).decode())
        out = dict(sums=sums, avn=avn.value, avs=avs.value, ext=ext, iposa=iposa)
        if streamfunctions:
            out.update(opsi=ops[0], opsip=ops[1], opsia=ops[2])
        return out

    @staticmethod
    def records(time: float, maxl: int, d: dict, opsisc: float = OPSISC):
        return format_records(time, maxl, d["sums"], d["avn"], d["avs"], d["ext"], d["iposa"], opsisc)


def format_records(time, maxl, sums, avn, avs, ext, iposa, opsisc=OPSISC):
    """(.t line, .s line, .opsit line) as step_goldstein writes them (gb_ts_format)."""
    lib = load_library()
    bufs = [C.create_string_buffer(256) for _ in range(3)]
    sums = np.ascontiguousarray(sums, dtype=np.float64)
    ext = np.ascontiguousarray(ext, dtype=np.float64)
    iposa = np.ascontiguousarray(iposa, dtype=np.int32)
    rc = lib.gb_ts_format(float(time), int(maxl), dptr(sums), float(avn), float(avs), dptr(ext),
                          iposa.ctypes.data_as(_ip), float(opsisc), bufs[0], bufs[1], bufs[2], 256)
    if rc != 0:
        raise GoldsteinError(rc, "gb_ts_format")
    return tuple(b.value.decode() for b in bufs)
