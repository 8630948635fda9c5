"""GOLDSTEIN restart files of a device-resident ocean (include/gb_restart.h).

Mirrors the reference's ``outm_netcdf(istep)`` and ``inm_netcdf(lrestart_genie)``
(src/goldstein/goldstein_data.f90:10-354): :func:`write_goldstein` writes the restart file of a
:class:`cgenie_gb300.goldstein.Goldstein` handle's current state (the temperature, salinity and
velocity fields are formed on the device, in the file's byte order), :func:`read_goldstein`
reads one back, and :func:`calendar_step` / :func:`calendar_after_read` keep the restart
calendar as the two routines do.  The files are netCDF classic (CDF-1) with outm_netcdf's
dimensions, variables and attributes.

3-D fields are C-order numpy arrays ``[k, j, i]`` (their memory is the Fortran
``(maxi, maxj, maxk)`` array), 2-D fields ``[j, i]``.
"""
from __future__ import annotations

import ctypes as C
from dataclasses import dataclass
from typing import Optional

import numpy as np

from . import abi
from .abi import dptr
from .goldstein import GoldsteinError, load_library


@dataclass
class Calendar:
    """iyear_rest, imonth_rest, ioffset_rest, day_rest and istep_ocn of goldstein_data.f90."""
    iyear: int = 0
    imonth: int = 1
    ioffset: int = 0
    day: float = 1.0
    istep: int = 0

    def to_c(self) -> abi.GbRsCalendar:
        return abi.GbRsCalendar(self.iyear, self.imonth, self.ioffset, self.istep, self.day)

    @staticmethod
    def from_c(c: abi.GbRsCalendar) -> "Calendar":
        return Calendar(c.iyear, c.imonth, c.ioffset, c.day, c.istep)


def _err(what: str, rc: int):
    raise GoldsteinError(rc, what, load_library().gb_rs_last_error().decode())


def _f64(a, shape) -> np.ndarray:
    a = np.ascontiguousarray(a, dtype=np.float64)
    if a.shape != tuple(shape):
        raise ValueError(f"expected shape {tuple(shape)}, got {a.shape}")
    return a


def write_goldstein(ocean, path: str, cal: Calendar, nclon1, nclat1, ncdepth, evap=None, late=None, sens=None,
                    gui: bool = False) -> None:
    """outm_netcdf's restart file of ``ocean``'s current state (no host copy of the tracers)."""
    d = ocean.m
    nclon1 = _f64(nclon1, (d.maxi,))
    nclat1 = _f64(nclat1, (d.maxj,))
    ncdepth = _f64(ncdepth, (d.maxk,))
    fl = [None if a is None else _f64(a, (d.maxj, d.maxi)) for a in (evap, late, sens)]
    c = cal.to_c()
    rc = load_library().gb_rs_write_goldstein(ocean.h, path.encode(), C.byref(c), int(bool(gui)), dptr(nclon1),
                                              dptr(nclat1), dptr(ncdepth), *(dptr(a) for a in fl))
    if rc:
        _err("gb_rs_write_goldstein", rc)


def pack_goldstein(ocean, dev_out: int) -> None:
    """The device part of a restart write: the four 3-D variables, big-endian, into the device
    buffer at address ``dev_out`` (4 * maxi*maxj*maxk doubles), enqueued on the ocean's stream."""
    rc = load_library().gb_rs_pack_goldstein(ocean.h, C.c_void_p(dev_out))
    if rc:
        _err("gb_rs_pack_goldstein", rc)


def write_fields(path: str, cal: Calendar, lon, lat, depths1, temp, salinity, uvel, vvel, evap=None, late=None,
                 sens=None, gui: bool = False) -> None:
    """The same file from host fields in file form (temp/salinity masked, depths1 bottom first)."""
    temp = np.ascontiguousarray(temp, dtype=np.float64)
    maxk, maxj, maxi = temp.shape
    f3 = [temp] + [_f64(a, temp.shape) for a in (salinity, uvel, vvel)]
    fl = [None if a is None else _f64(a, (maxj, maxi)) for a in (evap, late, sens)]
    ax = [_f64(lon, (maxi,)), _f64(lat, (maxj,)), _f64(depths1, (maxk,))]
    c = cal.to_c()
    rc = load_library().gb_rs_write_fields(path.encode(), maxi, maxj, maxk, C.byref(c), int(bool(gui)),
                                           *(dptr(a) for a in ax), *(dptr(a) for a in f3), *(dptr(a) for a in fl))
    if rc:
        _err("gb_rs_write_fields", rc)


_FIELDS = ("temp", "salinity", "uvel", "vvel", "evap", "late", "sens")


def read_goldstein(path: str, maxi: int, maxj: int, maxk: int, gui: bool = False, fields=_FIELDS):
    """inm_netcdf's read: (Calendar with day = iday as stored, dict of the requested fields)."""
    out = {n: np.zeros((maxk, maxj, maxi)) for n in ("temp", "salinity", "uvel", "vvel") if n in fields}
    out.update({n: np.zeros((maxj, maxi)) for n in ("evap", "late", "sens") if n in fields})
    c = abi.GbRsCalendar()
    rc = load_library().gb_rs_read_goldstein(path.encode(), maxi, maxj, maxk, int(bool(gui)), C.byref(c),
                                             *(dptr(out.get(n)) for n in _FIELDS))
    if rc:
        _err("gb_rs_read_goldstein", rc)
    return Calendar.from_c(c), out


def goldstein_name(dirnetout: str, cal: Calendar) -> str:
    """<dirnetout>/goldstein_restart_<iyear>_<mm>_<dd>.nc, as outm_netcdf names the file."""
    buf = C.create_string_buffer(len(dirnetout) + 64)
    c = cal.to_c()
    n = load_library().gb_rs_goldstein_name(dirnetout.encode(), C.byref(c), buf, len(buf))
    if n < 0:
        _err("gb_rs_goldstein_name", n)
    return buf.value.decode()


def calendar_step(cal: Calendar, yearlen: float, nyear: int) -> Calendar:
    """outm_netcdf's calendar advance (once per ocean step); returns the new calendar."""
    c = cal.to_c()
    load_library().gb_rs_calendar_step(C.byref(c), float(yearlen), int(nyear))
    return Calendar.from_c(c)


def calendar_after_read(cal: Calendar, yearlen: float, nyear: int) -> Calendar:
    """inm_netcdf's calendar update after its read; returns the new calendar."""
    c = cal.to_c()
    load_library().gb_rs_calendar_after_read(C.byref(c), float(yearlen), int(nyear))
    return Calendar.from_c(c)
