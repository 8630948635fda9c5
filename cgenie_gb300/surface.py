"""Device-resident 2-D surface steppers (include/gb_embm.h): the EMBM atmosphere step
``tstipa`` (src/embm/embm.f90:2039-2138) and the sea-ice transport step ``tstipsic``
(src/goldsteinseaice/gold_seaice.f90:937-1058).

Arrays are C-order numpy arrays whose memory is the reference's Fortran layout:
``tq[j, i, l]`` = tq(l+1, i+1, j+1) (2, maxi, maxj); ``pptn[j, i]`` = pptn(i+1, j+1);
``diffa[j, dir, l]`` = diffa(l+1, dir+1, j+1).
"""
from __future__ import annotations

import ctypes as C
from dataclasses import dataclass, field
from typing import Optional

import numpy as np

from . import abi
from .abi import dptr
from .goldstein import GoldsteinError, load_library


@dataclass
class SurfaceCase:
    """One surface grid's parameters, metrics, state and forcing."""
    kind: int
    maxi: int
    maxj: int
    maxk: int
    dt: float
    dphi: float
    rdphi: float
    rc: np.ndarray
    cv: np.ndarray
    dsv: np.ndarray
    rdsv: np.ndarray
    rds: np.ndarray
    tq: np.ndarray            # [j, i, 2]
    tq1: np.ndarray           # [j, i, 2]
    source: np.ndarray        # [j, i, 2]: tqa (EMBM) or dtha (sea ice)
    vel: np.ndarray           # [j, i, 2]: uatm (EMBM) or the surface ocean u(1:2) (sea ice)
    pptn: Optional[np.ndarray] = None    # [j, i] (EMBM)
    diffa: Optional[np.ndarray] = None   # [j, 2, 2] (EMBM)
    k1: Optional[np.ndarray] = None      # [0:maxj+1, 0:maxi+1] (sea ice)
    betaz: tuple = (1.0, 1.0)
    betam: tuple = (1.0, 1.0)
    diffmod0: float = 0.0
    ppmin: float = 0.0
    ppmax: float = 1.0
    diffsic: float = 0.0
    tsc: float = 0.0
    sica_thresh: float = 0.0
    sich_thresh: float = 0.0
    keep: list = field(default_factory=list)

    def params(self) -> abi.GbEaParams:
        return abi.GbEaParams(self.kind, self.maxk, self.dt, self.dphi, self.rdphi,
                              (C.c_double * 2)(*self.betaz), (C.c_double * 2)(*self.betam),
                              self.diffmod0, self.ppmin, self.ppmax, self.diffsic, self.tsc, self.sica_thresh,
                              self.sich_thresh)

    def grid(self) -> abi.GbEaGrid:
        arrs = [np.ascontiguousarray(a, dtype=np.float64) for a in (self.rc, self.cv, self.dsv, self.rdsv, self.rds)]
        diffa = None if self.diffa is None else np.ascontiguousarray(self.diffa, dtype=np.float64)
        k1 = None if self.k1 is None else np.ascontiguousarray(self.k1, dtype=np.int32)
        self.keep = arrs + [diffa, k1]
        return abi.GbEaGrid(*(dptr(a) for a in arrs), dptr(diffa),
                            None if k1 is None else k1.ctypes.data_as(C.POINTER(C.c_int32)))

    def copy(self) -> "SurfaceCase":
        import copy
        c = copy.copy(self)
        for n in ("tq", "tq1", "source", "vel", "pptn"):
            v = getattr(self, n)
            setattr(c, n, None if v is None else v.copy())
        c.keep = []
        return c


def embm_case(member, seed: int = 0, diffmod0: float = 0.0) -> SurfaceCase:
    """An EMBM step on a member's horizontal grid: seeded air temperature (deg C) and specific
    humidity, winds of a few m/s (nondimensional by usc = 0.05 m/s), diffusivities of a few
    1e6 m^2/s (nondimensional by rsc*usc), fluxes and precipitation with seeded noise."""
    rng = np.random.default_rng(seed)
    m = member
    mi, mj = m.maxi, m.maxj
    lat = np.linspace(-1.0, 1.0, mj)[:, None]
    T = 25.0 * (1.0 - lat ** 2) - 5.0 + rng.standard_normal((mj, mi))
    q = 0.015 * (1.0 - lat ** 2) + 1e-3 * rng.random((mj, mi))
    tq = np.stack([T, q], axis=-1)
    tq1 = tq + np.stack([0.1 * rng.standard_normal((mj, mi)), 1e-4 * rng.standard_normal((mj, mi))], axis=-1)
    usc, rsc = 0.05, 6.37e6
    vel = rng.standard_normal((mj, mi, 2)) * (5.0 / usc)
    diffa = np.empty((mj, 2, 2))
    diffa[:, 0, 0] = diffa[:, 1, 0] = 3.0e6 / (rsc * usc) * (1.0 + 0.5 * rng.random(mj))
    diffa[:, 0, 1] = diffa[:, 1, 1] = 1.0e6 / (rsc * usc) * (1.0 + 0.5 * rng.random(mj))
    source = np.stack([1e-2 * rng.standard_normal((mj, mi)), 1e-6 * rng.standard_normal((mj, mi))], axis=-1)
    pptn = 3e-8 * rng.random((mj, mi))
    return SurfaceCase(kind=abi.GB_EA_EMBM, maxi=mi, maxj=mj, maxk=m.maxk, dt=float(m.dt[0]) / 5.0,
                       dphi=m.dphi, rdphi=m.rdphi, rc=m.rc, cv=m.cv, dsv=m.dsv, rdsv=m.rdsv, rds=m.rds,
                       tq=tq, tq1=tq1, source=source, vel=vel, pptn=pptn, diffa=diffa,
                       betaz=(0.1, 0.9), betam=(0.0, 0.4), diffmod0=diffmod0, ppmin=1e-8, ppmax=2e-8)


def seaice_case(member, seed: int = 0, explicit: bool = False) -> SurfaceCase:
    """A sea-ice step on a member's grid and mask: ice height (m) and area fraction where the
    seeded surface is cold, the member's surface ocean velocities, seeded thermodynamic rates.
    explicit: the tstepsic form, with area/height thresholds (0.9, 2.5 m) that some cells pass."""
    rng = np.random.default_rng(seed)
    m = member
    mi, mj = m.maxi, m.maxj
    k1 = m.k1
    wet = k1[1:mj + 1, 1:mi + 1] <= m.maxk
    lat = np.abs(np.linspace(-1.0, 1.0, mj))[:, None]
    cold = np.clip((lat - 0.5) * 2.0, 0.0, 1.0) * np.ones((1, mi))
    H = np.where(wet, 3.0 * cold * rng.random((mj, mi)), 0.0)
    A = np.where(wet, np.clip(cold + 0.1 * rng.standard_normal((mj, mi)), 0.0, 1.0), 0.0)
    tq = np.stack([H, A], axis=-1)
    tq1 = tq.copy()
    top = m.u[m.maxk - 1]                # u(3, 0:maxi, 0:maxj, maxk) as [j, i, c]
    vel = np.ascontiguousarray(top[1:mj + 1, 1:mi + 1, :2])
    usc, rsc = 0.05, 6.37e6
    tsc = rsc / usc
    source = np.where(wet[..., None], 1e-9 * rng.standard_normal((mj, mi, 2)), 0.0)
    return SurfaceCase(kind=abi.GB_EA_SEAICE_EXPLICIT if explicit else abi.GB_EA_SEAICE, maxi=mi, maxj=mj,
                       maxk=m.maxk, dt=float(m.dt[0]), dphi=m.dphi, rdphi=m.rdphi, rc=m.rc, cv=m.cv, dsv=m.dsv,
                       rdsv=m.rdsv, rds=m.rds, tq=tq, tq1=tq1, source=source, vel=vel, k1=k1,
                       diffsic=2000.0 / (rsc * usc), tsc=tsc, sica_thresh=0.9, sich_thresh=2.5)


def seaice_post_constants(case: SurfaceCase) -> abi.GbEaSeaicePost:
    """The reference's post-processing constants for a sea-ice case: rhoio = rhoice/rho0,
    rhoice = 913, rho0 = 1000, hmin = 0.01 (gold_seaice_lib.f90:33-34; gold_seaice.f90:304),
    rdtdim = 1/(tsc*dtsic) (gold_seaice.f90:262), hlf = 3.34e5 (gold_seaice_lib.f90:38), m2mm = 1000."""
    return abi.GbEaSeaicePost(rhoio=913.0 / 1.0e3, rhoice=913.0, hlf=3.34e5, hmin=0.01,
                              rdtdim=1.0 / (case.tsc * case.dt), m2mm=1000.0)


class SurfaceStepper:
    """A device-resident surface grid (gb_ea handle)."""

    def __init__(self, case: SurfaceCase, device: int = -1):
        self.lib = load_library()
        self.case = case
        self.dims = abi.GbEaDims(case.maxi, case.maxj)
        self.params = case.params()
        self.grid = case.grid()
        h = C.c_void_p()
        rc = self.lib.gb_ea_create(C.byref(self.dims), C.byref(self.params), C.byref(self.grid), int(device),
                                   C.byref(h))
        if rc != 0:
            raise GoldsteinError(rc, "gb_ea_create")
        self.h = h

    def _check(self, rc: int, what: str):
        if rc != 0:
            detail = self.lib.gb_ea_last_error(self.h).decode() if self.h else ""
            raise GoldsteinError(rc, what, detail)

    def close(self):
        if self.h:
            self.lib.gb_ea_destroy(self.h)
            self.h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def upload_state(self, tq=None, tq1=None):
        c = self.case
        tq = np.ascontiguousarray(c.tq if tq is None else tq, dtype=np.float64)
        tq1 = np.ascontiguousarray(c.tq1 if tq1 is None else tq1, dtype=np.float64)
        self._check(self.lib.gb_ea_upload_state(self.h, dptr(tq), dptr(tq1)), "gb_ea_upload_state")

    def set_forcing(self, source=None, vel=None, pptn=None):
        c = self.case
        s = np.ascontiguousarray(c.source if source is None else source, dtype=np.float64)
        v = np.ascontiguousarray(c.vel if vel is None else vel, dtype=np.float64)
        p = c.pptn if pptn is None else pptn
        p = None if p is None else np.ascontiguousarray(p, dtype=np.float64)
        self._check(self.lib.gb_ea_set_forcing(self.h, dptr(s), dptr(v), dptr(p)), "gb_ea_set_forcing")

    def step(self, nsteps: int = 1):
        self._check(self.lib.gb_ea_step(self.h, int(nsteps)), "gb_ea_step")

    def download(self):
        c = self.case
        tq = np.zeros((c.maxj, c.maxi, 2))
        tq1 = np.zeros((c.maxj, c.maxi, 2))
        self._check(self.lib.gb_ea_download(self.h, dptr(tq), dptr(tq1)), "gb_ea_download")
        return tq, tq1

    def set_seaice_post(self, post: Optional[abi.GbEaSeaicePost]):
        """Post-process every sea-ice step as step_seaice does (gold_seaice.f90:599-619), or
        stop (None); with it on, step(n) takes n step_seaice steps."""
        self._check(self.lib.gb_ea_set_seaice_post(self.h, None if post is None else C.byref(post)),
                    "gb_ea_set_seaice_post")

    def download_seaice_fluxes(self):
        """(fx_delta, fw_delta) [j, i] of the last post-processed step."""
        c = self.case
        fx = np.zeros((c.maxj, c.maxi))
        fw = np.zeros((c.maxj, c.maxi))
        self._check(self.lib.gb_ea_download_seaice_fluxes(self.h, dptr(fx), dptr(fw)), "gb_ea_download_seaice_fluxes")
        return fx, fw

    def download_seaice_diag(self):
        """(variceth, varicedy) [j, i, l] of the last tstipsic step (gold_seaice.f90:1046-1056)."""
        c = self.case
        th = np.zeros((c.maxj, c.maxi, 2))
        dy = np.zeros((c.maxj, c.maxi, 2))
        self._check(self.lib.gb_ea_download_seaice_diag(self.h, dptr(th), dptr(dy)), "gb_ea_download_seaice_diag")
        return th, dy


def step_many(steppers, nsteps: int = 1):
    """One launch advancing every stepper (same kind and shape, one device) by nsteps."""
    if not steppers:
        return
    lib = steppers[0].lib
    arr = (C.c_void_p * len(steppers))(*[s.h for s in steppers])
    rc = lib.gb_ea_step_many(arr, len(steppers), int(nsteps))
    if rc != 0:
        steppers[0]._check(rc, "gb_ea_step_many")
