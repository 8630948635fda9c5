"""Oracle (test infrastructure only): a NumPy / pure-Python restatement of the GOLDSTEIN restart
routines outm_netcdf and inm_netcdf (src/goldstein/goldstein_data.f90:10-354).

It restates what goes into the restart file (the masked tracer fields, the velocities, the
reversed depth axis, the calendar scalars), the file name and the calendar updates.  The file
encoding itself is checked against an independent netCDF classic reader and the netCDF-written
file the reference ships (data/main/main_restart_0.nc, a CDF-1 file of the same scalar
variables), so this module holds no codec.  Only tests and the smoke check use it.

Array layouts are those of cgenie_gb300.grid: ts (maxk+2, maxj+2, maxi+2, maxl) = Fortran
ts(l, 0:maxi+1, 0:maxj+1, 0:maxk+1); u (maxk, maxj+1, maxi+1, 3) = u(3, 0:maxi, 0:maxj, 1:maxk);
k1 (maxj+2, maxi+2) = k1(0:maxi+1, 0:maxj+1).  Fields come out as [k, j, i].
"""
from __future__ import annotations

import math

import numpy as np


def restart_fields(ts: np.ndarray, u: np.ndarray, k1: np.ndarray, maxi: int, maxj: int, maxk: int):
    """temp, salinity, uvel, vvel as outm_netcdf writes them (goldstein_data.f90:194-213).

    landmask(i, j, :) = 1 for every level of a column as soon as one level k in 1..maxk has
    k >= k1(i, j) (:200-206), i.e. on the whole of each wet column; temp and salinity are
    ts * landmask in double precision (-0.0 for negative values on land, as the product gives).
    """
    k1i = k1[1:maxj + 1, 1:maxi + 1]
    landmask = (k1i <= maxk).astype(np.float64)[None, :, :]
    temp = ts[1:maxk + 1, 1:maxj + 1, 1:maxi + 1, 0] * landmask
    sal = ts[1:maxk + 1, 1:maxj + 1, 1:maxi + 1, 1] * landmask
    uvel = np.array(u[:, 1:maxj + 1, 1:maxi + 1, 0])
    vvel = np.array(u[:, 1:maxj + 1, 1:maxi + 1, 1])
    return temp, sal, uvel, vvel


def depths1(ncdepth: np.ndarray) -> np.ndarray:
    """depths1(k) = ncdepth(maxk-k+1) (:196-198), stored as NF90_REAL (float32)."""
    return np.asarray(ncdepth, dtype=np.float64)[::-1].astype(np.float32)


def nint(x: float) -> int:
    """Fortran NINT: the nearest integer, halves away from zero."""
    a = abs(x)
    r = math.floor(a)
    if a - r >= 0.5:   # exact for doubles below 2**52
        r += 1
    return int(r) if x >= 0 else -int(r)


def goldstein_name(dirnetout: str, iyear: int, imonth: int, day: float) -> str:
    """TRIM(dirnetout)//'/goldstein_restart_'//yearstring//'_'//mm//'_'//dd//'.nc' (:216-227)
    with the edit descriptors i10 (adjusted left, trimmed) and i2.2 (asterisks when the value
    does not fit)."""
    y = str(iyear)
    if len(y) > 10:
        y = "*" * 10
    iday = nint(day)
    mm = "%02d" % imonth if 0 <= imonth <= 99 else "**"
    dd = "%02d" % iday if 0 <= iday <= 99 else "**"
    return f"{dirnetout.rstrip()}/goldstein_restart_{y}_{mm}_{dd}.nc"


def _roll(day: float, imonth: int, iyear: int):
    if day >= 31:
        day = day - 30
        imonth = imonth + 1
        if imonth == 13:
            imonth = 1
            iyear = iyear + 1
    return day, imonth, iyear


def calendar_step(iyear: int, imonth: int, day: float, yearlen: float, nyear: int):
    """The calendar lines of outm_netcdf (:185-188 and :320-338): (iyear, imonth, day)."""
    timestep = yearlen / float(nyear)
    iday = nint(day)
    day = day + timestep
    if abs(iday - day) <= 1.0e-3:
        day = float(iday)
    day, imonth, iyear = _roll(day, imonth, iyear)
    return iyear, imonth, day


def calendar_after_read(iyear: int, imonth: int, ioffset: int, iday: int, yearlen: float, nyear: int):
    """The calendar lines of inm_netcdf after its read (:32, :70-85): (iyear, imonth, ioffset,
    day).  MOD keeps the sign of the dividend, as math.fmod does."""
    timestep = 24.0 * 60.0 * 60.0 * yearlen / float(nyear)
    day = float(iday)
    n = nint(yearlen)
    ioffset = int(math.fmod(ioffset, n)) if n != 0 else ioffset
    day = day + timestep / (24 * 60 * 60.0)
    if abs(iday - day) <= 1.0e-3:
        day = float(iday)
    day, imonth, iyear = _roll(day, imonth, iyear)
    return iyear, imonth, ioffset, day
