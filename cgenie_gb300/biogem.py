"""BIOGEM tracer coupling on the device (include/gb_biogem.h).

Mirrors the reference's ``biogem_tracercoupling(go_ts, go_ts1)``
(src/biogem/biogem.f90:1885-2077): BIOGEM's vector fields (``vocn``, ``vphys_ocn`` masses,
volumes and reciprocal masses, ``vbio_part``) and the interval's increments (``vdocn``,
``vdbio_part``) live on the device; :meth:`BiogemCoupling.tracercoupling` applies the
coupling to the tracer state of a :class:`cgenie_gb300.goldstein.Goldstein` handle in place.

Arrays use the reference's vector form (src/biogem/biogem_lib.f90:1056-1081) as C-order
numpy arrays whose memory is the Fortran packing of include/gb_biogem.h:
``vocn[n, k, l]`` = vocn(n+1)%mk(l+1, k+1), ``mass[n, k]`` = vphys_ocn(n+1)%mk(ipo_M, k+1),
with n running over the wet columns, i outer and j inner.
"""
from __future__ import annotations

import ctypes as C
from dataclasses import dataclass
from typing import Optional

import numpy as np

from . import abi
from .abi import dptr
from .goldstein import GoldsteinError, load_library

CONST_ZEROC = 273.15      # const_zeroC (src/common/gem_cmn.f90), tstoocn_offset(1)
SALN0 = 34.9              # goldstein_saln0 default (goldstein-defaults.nml), tstoocn_offset(2)


def wet_columns(k1_interior: np.ndarray, n_k: int):
    """(i, j, k1) of the wet columns in vector order; k1_interior is [j, i] (C order) of
    goldstein_k1(1:n_i, 1:n_j)."""
    n_j, n_i = k1_interior.shape
    return [(i, j, int(k1_interior[j, i])) for i in range(n_i) for j in range(n_j) if k1_interior[j, i] <= n_k]


@dataclass
class BiogemState:
    """BIOGEM's vector fields of one grid (see the module docstring for the layout)."""
    vocn: np.ndarray          # (nv, n_k, n_l_ocn)
    mass: np.ndarray          # (nv, n_k)
    volume: np.ndarray        # (nv, n_k)
    rmass: np.ndarray         # (nv, n_k)
    vbio_part: np.ndarray     # (nv, n_k, n_l_sed)
    vdocn: np.ndarray         # (nv, n_k, n_l_ocn)
    vdbio_part: np.ndarray    # (nv, n_k, n_l_sed)

    def copy(self) -> "BiogemState":
        return BiogemState(*(np.array(a, copy=True) for a in (self.vocn, self.mass, self.volume, self.rmass,
                                                              self.vbio_part, self.vdocn, self.vdbio_part)))


def make_state(member, n_l_sed: int = 4, seed: int = 0, increments: float = 1.0,
               ts_offset=(CONST_ZEROC, SALN0)) -> BiogemState:
    """Seeded BIOGEM fields consistent with a member's GOLDSTEIN tracers: vocn(T, S) are the
    member's T and S plus the offsets, the biogeochemical tracers are the member's tracers
    de-normalised by S / mean S; volumes are the member's cell volumes in m^3 (grid metrics
    times the reference's scales), masses volume x 1027.649 kg/m^3 with small seeded
    variation; increments of about 1e-4 (T, S) and 1e-3 relative (others), times `increments`."""
    rng = np.random.default_rng(seed)
    m = member
    nk, L = m.maxk, m.maxl
    k1 = m.k1[1:m.maxj + 1, 1:m.maxi + 1]
    cols = wet_columns(k1, nk)
    nv = len(cols)
    rsc, dsc = 6.37e6, 5.0e3
    vocn = np.zeros((nv, nk, L))
    volume = np.zeros((nv, nk))
    wet = np.zeros((nv, nk), bool)
    for n, (i, j, kk) in enumerate(cols):
        wet[n, kk - 1:] = True
        vocn[n, kk - 1:, :] = m.ts[kk:nk + 1, j + 1, i + 1, :]
        area = m.dphi * m.ds[j] * rsc * rsc
        volume[n, kk - 1:] = area * m.dz[kk - 1:nk] * dsc
    vocn[..., 0] += ts_offset[0]
    vocn[..., 1] += ts_offset[1]
    if L > 2:
        s = vocn[..., 1]
        mean_s = float((s * volume)[wet].sum() / volume[wet].sum())
        vocn[..., 2:] *= (s / mean_s)[..., None]
    vocn[~wet] = 0.0
    mass = np.where(wet, volume * 1027.649 * (1.0 + 1e-3 * rng.standard_normal((nv, nk))), 0.0)
    rmass = np.where(wet, 1.0 / np.where(wet, mass, 1.0), 0.0)
    vbio = np.where(wet[..., None], np.exp(rng.standard_normal((nv, nk, n_l_sed))), 0.0)
    vd = np.zeros_like(vocn)
    vd[..., 0] = 1e-4 * rng.standard_normal((nv, nk))
    vd[..., 1] = 1e-4 * rng.standard_normal((nv, nk))
    if L > 2:
        vd[..., 2:] = 1e-3 * np.abs(vocn[..., 2:]) * rng.standard_normal((nv, nk, L - 2))
    vd = np.where(wet[..., None], increments * vd, 0.0)
    vdb = np.where(wet[..., None], increments * 1e-3 * rng.standard_normal((nv, nk, n_l_sed)), 0.0)
    return BiogemState(vocn, mass, volume, rmass, vbio, vd, vdb)


class BiogemCoupling:
    """Device-resident BIOGEM fields of one grid and the tracer coupling."""

    def __init__(self, member, *, n_l_sed: int = 4, ts_offset=(CONST_ZEROC, SALN0), force_ts: bool = False,
                 device: int = -1):
        self.lib = load_library()
        m = member
        self.dims = abi.GbBgDims(m.maxi, m.maxj, m.maxk, m.maxl, n_l_sed, 0)
        self.params = abi.GbBgParams((C.c_double * 2)(*ts_offset), int(bool(force_ts)), 0)
        # goldstein_k1(1:n_i, 1:n_j), i fastest
        self._k1 = np.ascontiguousarray(m.k1[1:m.maxj + 1, 1:m.maxi + 1], dtype=np.int32)
        h = C.c_void_p()
        rc = self.lib.gb_bg_create(C.byref(self.dims), C.byref(self.params),
                                   self._k1.ctypes.data_as(C.POINTER(C.c_int32)), int(device), C.byref(h))
        if rc != 0:
            raise GoldsteinError(rc, "gb_bg_create")
        self.h = h
        self.nv = int(self.lib.gb_bg_columns(self.h))
        self.n_k, self.L, self.Ls = m.maxk, m.maxl, n_l_sed

    def _check(self, rc: int, what: str):
        if rc != 0:
            detail = self.lib.gb_bg_last_error(self.h).decode() if self.h else ""
            raise GoldsteinError(rc, what, detail)

    def close(self):
        if self.h:
            self.lib.gb_bg_destroy(self.h)
            self.h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    @staticmethod
    def _arr(a: Optional[np.ndarray]):
        if a is None:
            return None
        a = np.ascontiguousarray(a, dtype=np.float64)
        return a

    def upload(self, st: BiogemState):
        """vocn, masses, volumes, reciprocal masses, particulates."""
        arrs = [self._arr(a) for a in (st.vocn, st.mass, st.volume, st.rmass, st.vbio_part)]
        self._check(self.lib.gb_bg_upload(self.h, *[dptr(a) if a is not None and a.size else None for a in arrs]),
                    "gb_bg_upload")

    def set_increments(self, st: BiogemState):
        a, b = self._arr(st.vdocn), self._arr(st.vdbio_part)
        self._check(self.lib.gb_bg_set_increments(self.h, dptr(a), dptr(b) if b.size else None),
                    "gb_bg_set_increments")

    def tracercoupling(self, ocean):
        """biogem_tracercoupling(go_ts, go_ts1) on the device state of `ocean` (a Goldstein handle)."""
        self._check(self.lib.gb_bg_tracercoupling(self.h, ocean.h), "gb_bg_tracercoupling")

    def download(self):
        """(vocn, mass, rmass, vbio_part) after the coupling."""
        vocn = np.zeros((self.nv, self.n_k, self.L))
        mass = np.zeros((self.nv, self.n_k))
        rmass = np.zeros((self.nv, self.n_k))
        vbio = np.zeros((self.nv, self.n_k, self.Ls))
        self._check(self.lib.gb_bg_download(self.h, dptr(vocn), dptr(mass), dptr(rmass),
                                            dptr(vbio) if vbio.size else None), "gb_bg_download")
        return vocn, mass, rmass, vbio
