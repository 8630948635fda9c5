"""Host-side mirror of the reference's tracer-step interface over the C-ABI.

The reference calls ``CALL tstepo`` (src/goldstein/goldstein.f90:235) on SAVE'd
module arrays; :class:`Goldstein` holds the same arrays (``ts``, ``ts1``,
``rho``, ``u``, ``cost``, ``icosd`` in Fortran layout) and forwards them to
libgb_goldstein.so, where the state stays resident on the GPU between
``tstepo()`` calls and is copied back only by :meth:`Goldstein.download` (the
coupling-interval copy of goldstein.f90:443-450).

There is no CPU fallback: importing works without a GPU, but creating a
:class:`Goldstein` requires the CUDA library and a device, and raises otherwise.
"""
from __future__ import annotations

import ctypes as C
import os
from typing import Optional

import numpy as np

from . import abi
from .abi import GbDims, GbEnsTuning, GbGrid, GbParams, GridRefs, dptr, iptr

HERE = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(HERE, "_lib", "libgb_goldstein.so")

# every exported entry point of include/gb_goldstein.h
EXPORTED = [
    "gb_go_create", "gb_go_destroy", "gb_go_set_stream", "gb_go_upload_state", "gb_go_set_forcing",
    "gb_go_set_velocity", "gb_go_set_diag", "gb_go_tstepo", "gb_go_download", "gb_go_inventory",
    "gb_go_inventory_noalloc", "gb_go_set_mld_wind", "gb_go_download_mld",
    "gb_go_sync", "gb_go_errstr", "gb_go_last_error", "gb_go_kernel_launch_count",
    "gb_ens_create", "gb_ens_destroy", "gb_ens_set_tuning", "gb_ens_set_stream", "gb_ens_member_bytes",
    "gb_ens_add", "gb_ens_add_many", "gb_ens_remove", "gb_ens_step", "gb_ens_set_remaining", "gb_ens_step_remaining",
    "gb_ens_remaining", "gb_ens_download", "gb_ens_download_many", "gb_ens_download_stream", "gb_ens_inventory", "gb_ens_status", "gb_ens_sync",
    "gb_ens_count", "gb_ens_last_error", "gb_ens_host_alloc", "gb_ens_host_free", "gb_ens_set_mld_wind",
    "gb_ens_download_mld",
    "gb_bg_create", "gb_bg_destroy", "gb_bg_columns", "gb_bg_upload", "gb_bg_set_increments",
    "gb_bg_tracercoupling", "gb_bg_download", "gb_bg_last_error",
    "gb_ea_create", "gb_ea_destroy", "gb_ea_upload_state", "gb_ea_set_forcing", "gb_ea_step", "gb_ea_step_many",
    "gb_ea_download",
    "gb_ea_download_seaice_diag",
    "gb_ea_set_seaice_post",
    "gb_ea_download_seaice_fluxes",
    "gb_ea_last_error",
    "gb_mo_create", "gb_mo_destroy", "gb_mo_set_wind", "gb_mo_upload_velocity", "gb_mo_step", "gb_mo_download",
    "gb_mo_last_error",
    "gb_rs_write_goldstein", "gb_rs_pack_goldstein", "gb_rs_write_fields", "gb_rs_read_goldstein", "gb_rs_goldstein_name",
    "gb_rs_calendar_step", "gb_rs_calendar_after_read", "gb_rs_last_error",
    "gb_ts_create", "gb_ts_destroy", "gb_ts_diagnose", "gb_ts_format", "gb_ts_last_error",
    "gb_tr_resume", "gb_tr_pause", "gb_tr_domain_create", "gb_tr_string_handle_create", "gb_tr_task_begin",
    "gb_tr_task_end",
]

_lib = None


class GoldsteinError(RuntimeError):
    def __init__(self, code: int, what: str, detail: str = ""):
        self.code = code
        name = abi.ERRNAMES.get(code, str(code))
        super().__init__(f"{what} failed: {name} ({code}) {detail}".rstrip())


def load_library(path: str = LIB_PATH):
    """Load libgb_goldstein.so (built by cgenie_gb300.build).  Raises if absent."""
    global _lib
    if _lib is not None:
        return _lib
    if not os.path.exists(path):
        raise RuntimeError(f"CUDA library not built: {path} (run `python -m cgenie_gb300.build`)")
    L = C.CDLL(path)
    P = C.POINTER
    vp = C.c_void_p
    dp = P(C.c_double)
    ip = P(C.c_int32)
    L.gb_go_create.argtypes = [P(GbDims), P(GbParams), P(GbGrid), C.c_int, P(vp)]
    L.gb_go_destroy.argtypes = [vp]
    L.gb_go_destroy.restype = None
    L.gb_go_set_stream.argtypes = [vp, vp]
    L.gb_go_upload_state.argtypes = [vp, dp, dp, dp]
    L.gb_go_set_forcing.argtypes = [vp, dp]
    L.gb_go_set_velocity.argtypes = [vp, dp]
    L.gb_go_set_diag.argtypes = [vp, dp, ip]
    L.gb_go_tstepo.argtypes = [vp, C.c_int32]
    L.gb_go_download.argtypes = [vp, dp, dp, dp, dp, ip, dp, ip]
    L.gb_go_inventory.argtypes = [vp, dp]
    L.gb_go_inventory_noalloc.argtypes = [vp, dp]
    L.gb_go_set_mld_wind.argtypes = [vp, dp]
    L.gb_go_download_mld.argtypes = [vp, dp, ip]
    L.gb_go_sync.argtypes = [vp]
    L.gb_go_errstr.argtypes = [C.c_int]
    L.gb_go_errstr.restype = C.c_char_p
    L.gb_go_last_error.argtypes = [vp]
    L.gb_go_last_error.restype = C.c_char_p
    L.gb_go_kernel_launch_count.argtypes = []
    L.gb_go_kernel_launch_count.restype = C.c_uint64
    L.gb_ens_create.argtypes = [C.c_int, C.c_size_t, P(vp)]
    L.gb_ens_destroy.argtypes = [vp]
    L.gb_ens_destroy.restype = None
    L.gb_ens_set_tuning.argtypes = [vp, P(GbEnsTuning)]
    L.gb_ens_set_stream.argtypes = [vp, vp]
    L.gb_ens_member_bytes.argtypes = [P(GbDims), P(GbParams)]
    L.gb_ens_member_bytes.restype = C.c_size_t
    L.gb_ts_create.argtypes = [P(GbDims), P(GbGrid), vp, C.c_int, P(vp)]
    L.gb_ts_destroy.argtypes = [vp]
    L.gb_ts_destroy.restype = None
    L.gb_ts_diagnose.argtypes = [vp, vp, dp, dp, dp, dp, ip, dp, dp, dp]
    L.gb_ts_format.argtypes = [C.c_double, C.c_int32, dp, C.c_double, C.c_double, dp, ip, C.c_double,
                               C.c_char_p, C.c_char_p, C.c_char_p, C.c_int32]
    L.gb_ts_last_error.argtypes = [vp]
    L.gb_ts_last_error.restype = C.c_char_p
    L.gb_tr_resume.argtypes = []
    L.gb_tr_pause.argtypes = []
    L.gb_tr_domain_create.argtypes = [C.c_char_p]
    L.gb_tr_domain_create.restype = vp
    L.gb_tr_string_handle_create.argtypes = [C.c_char_p]
    L.gb_tr_string_handle_create.restype = vp
    L.gb_tr_task_begin.argtypes = [vp, vp]
    L.gb_tr_task_begin.restype = None
    L.gb_tr_task_end.argtypes = [vp]
    L.gb_tr_task_end.restype = None
    L.gb_ens_add.argtypes = [vp, P(GbDims), P(GbParams), P(GbGrid), dp, dp, ip]
    L.gb_ens_add_many.argtypes = [vp, C.c_int32, P(GbDims), P(GbParams), P(GbGrid), P(vp), P(vp), ip]
    L.gb_ens_remove.argtypes = [vp, C.c_int32]
    L.gb_ens_step.argtypes = [vp, C.c_int32]
    L.gb_ens_set_remaining.argtypes = [vp, C.c_int32, C.c_int64]
    L.gb_ens_step_remaining.argtypes = [vp, C.c_int32]
    L.gb_ens_remaining.argtypes = [vp, C.c_int32, P(C.c_int64)]
    L.gb_ens_download.argtypes = [vp, C.c_int32, dp, dp, dp]
    L.gb_ens_download_stream.argtypes = [vp, C.c_int32, vp, dp, dp, dp]
    L.gb_ens_download_many.argtypes = [vp, C.c_int32, ip, P(dp), P(dp), P(dp)]
    L.gb_ens_inventory.argtypes = [vp, C.c_int32, dp]
    L.gb_ens_status.argtypes = [vp, C.c_int32, ip]
    L.gb_ens_sync.argtypes = [vp]
    L.gb_ens_count.argtypes = [vp, ip, P(C.c_size_t)]
    L.gb_ens_last_error.argtypes = [vp]
    L.gb_ens_last_error.restype = C.c_char_p
    L.gb_ens_host_alloc.argtypes = [C.c_size_t, P(vp)]
    L.gb_ens_set_mld_wind.argtypes = [vp, C.c_int32, dp]
    L.gb_ens_download_mld.argtypes = [vp, C.c_int32, dp, ip]
    L.gb_ens_host_free.argtypes = [vp]
    L.gb_bg_create.argtypes = [P(abi.GbBgDims), P(abi.GbBgParams), ip, C.c_int, P(vp)]
    L.gb_bg_destroy.argtypes = [vp]
    L.gb_bg_destroy.restype = None
    L.gb_bg_columns.argtypes = [vp]
    L.gb_bg_columns.restype = C.c_int32
    L.gb_bg_upload.argtypes = [vp, dp, dp, dp, dp, dp]
    L.gb_bg_set_increments.argtypes = [vp, dp, dp]
    L.gb_bg_tracercoupling.argtypes = [vp, vp]
    L.gb_bg_download.argtypes = [vp, dp, dp, dp, dp]
    L.gb_bg_last_error.argtypes = [vp]
    L.gb_bg_last_error.restype = C.c_char_p
    L.gb_ea_create.argtypes = [P(abi.GbEaDims), P(abi.GbEaParams), P(abi.GbEaGrid), C.c_int, P(vp)]
    L.gb_ea_destroy.argtypes = [vp]
    L.gb_ea_destroy.restype = None
    L.gb_ea_upload_state.argtypes = [vp, dp, dp]
    L.gb_ea_set_forcing.argtypes = [vp, dp, dp, dp]
    L.gb_ea_step.argtypes = [vp, C.c_int32]
    L.gb_ea_step_many.argtypes = [P(vp), C.c_int32, C.c_int32]
    L.gb_ea_download.argtypes = [vp, dp, dp]
    L.gb_ea_download_seaice_diag.argtypes = [vp, dp, dp]
    L.gb_ea_set_seaice_post.argtypes = [vp, C.POINTER(abi.GbEaSeaicePost)]
    L.gb_ea_download_seaice_fluxes.argtypes = [vp, dp, dp]
    L.gb_ea_last_error.argtypes = [vp]
    L.gb_ea_last_error.restype = C.c_char_p
    L.gb_mo_create.argtypes = [vp, vp, vp, C.c_int, P(vp)]
    L.gb_mo_destroy.argtypes = [vp]
    L.gb_mo_destroy.restype = None
    L.gb_mo_set_wind.argtypes = [vp, dp, dp, dp]
    L.gb_mo_upload_velocity.argtypes = [vp, dp, dp]
    L.gb_mo_step.argtypes = [vp, vp]
    L.gb_mo_download.argtypes = [vp, dp, dp, dp, dp]
    L.gb_mo_last_error.argtypes = [vp]
    L.gb_mo_last_error.restype = C.c_char_p
    L.gb_rs_write_goldstein.argtypes = [vp, C.c_char_p, vp, C.c_int32, dp, dp, dp, dp, dp, dp]
    L.gb_rs_pack_goldstein.argtypes = [vp, vp]
    L.gb_rs_write_fields.argtypes = [C.c_char_p, C.c_int32, C.c_int32, C.c_int32, vp, C.c_int32,
                                     dp, dp, dp, dp, dp, dp, dp, dp, dp, dp]
    L.gb_rs_read_goldstein.argtypes = [C.c_char_p, C.c_int32, C.c_int32, C.c_int32, C.c_int32, vp,
                                       dp, dp, dp, dp, dp, dp, dp]
    L.gb_rs_goldstein_name.argtypes = [C.c_char_p, vp, C.c_char_p, C.c_int32]
    L.gb_rs_calendar_step.argtypes = [vp, C.c_double, C.c_int32]
    L.gb_rs_calendar_step.restype = None
    L.gb_rs_calendar_after_read.argtypes = [vp, C.c_double, C.c_int32]
    L.gb_rs_calendar_after_read.restype = None
    L.gb_rs_last_error.argtypes = []
    L.gb_rs_last_error.restype = C.c_char_p
    _lib = L
    return L


def kernel_launch_count() -> int:
    return int(load_library().gb_go_kernel_launch_count())


class Goldstein:
    """One GOLDSTEIN grid with device-resident tracer state.

    Mirrors the reference's call sequence in step_goldstein
    (goldstein.f90:167-187, 235, 443-450): set the forcing slot and the
    velocities, call :meth:`tstepo`, and copy back at coupling intervals.
    """

    def __init__(self, member, *, precision: int = abi.GB_GO_FP64, device: int = -1,
                 diso=None, ieos=None, iconv=None, iediff=None, imld=None, stream: Optional[int] = None):
        self.lib = load_library()
        self.m = member
        self.refs = GridRefs(member, diso=diso, ieos=ieos, iconv=iconv, iediff=iediff, imld=imld,
                             precision=precision)
        h = C.c_void_p()
        rc = self.lib.gb_go_create(C.byref(self.refs.dims), C.byref(self.refs.params), C.byref(self.refs.grid),
                                   int(device), C.byref(h))
        if rc != 0:
            raise GoldsteinError(rc, "gb_go_create")
        self.h = h
        if stream is not None:
            self._check(self.lib.gb_go_set_stream(self.h, C.c_void_p(stream)), "gb_go_set_stream")

    # -- plumbing
    def _check(self, rc: int, what: str):
        if rc != 0:
            detail = self.lib.gb_go_last_error(self.h).decode() if self.h else ""
            raise GoldsteinError(rc, what, detail)

    def close(self):
        if getattr(self, "h", None):
            self.lib.gb_go_destroy(self.h)
            self.h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def set_stream(self, stream: Optional[int]):
        self._check(self.lib.gb_go_set_stream(self.h, C.c_void_p(stream or 0)), "gb_go_set_stream")

    # -- the reference's data movement
    def upload_state(self, ts=None, ts1=None, rho=None):
        m = self.m
        ts = np.ascontiguousarray(m.ts if ts is None else ts, dtype=np.float64)
        ts1 = np.ascontiguousarray(m.ts1 if ts1 is None else ts1, dtype=np.float64)
        rho = np.ascontiguousarray(m.rho if rho is None else rho, dtype=np.float64)
        self._check(self.lib.gb_go_upload_state(self.h, dptr(ts), dptr(ts1), dptr(rho)), "gb_go_upload_state")

    def set_forcing(self, top):
        top = np.ascontiguousarray(top, dtype=np.float64)
        self._check(self.lib.gb_go_set_forcing(self.h, dptr(top)), "gb_go_set_forcing")

    def set_velocity(self, u=None):
        u = np.ascontiguousarray(self.m.u if u is None else u, dtype=np.float64)
        self._check(self.lib.gb_go_set_velocity(self.h, dptr(u)), "gb_go_set_velocity")

    def set_diag(self, cost=None, icosd=None):
        c = None if cost is None else np.ascontiguousarray(cost, dtype=np.float64)
        i = None if icosd is None else np.ascontiguousarray(icosd, dtype=np.int32)
        self._check(self.lib.gb_go_set_diag(self.h, dptr(c), iptr(i)), "gb_go_set_diag")

    def tstepo(self, nsteps: int = 1):
        self._check(self.lib.gb_go_tstepo(self.h, int(nsteps)), "gb_go_tstepo")

    def sync(self):
        self._check(self.lib.gb_go_sync(self.h), "gb_go_sync")

    def download(self):
        """Return dict(ts, ts1, rho, cost, icosd, dmax, limps) in Fortran layout."""
        m = self.m
        ts = np.empty_like(m.ts)
        ts1 = np.empty_like(m.ts1)
        rho = np.empty_like(m.rho)
        cost = np.empty_like(m.cost)
        icosd = np.empty_like(m.icosd)
        dmax = C.c_double()
        limps = C.c_int32()
        self._check(self.lib.gb_go_download(self.h, dptr(ts), dptr(ts1), dptr(rho), dptr(cost), iptr(icosd),
                                            C.byref(dmax), C.byref(limps)), "gb_go_download")
        return dict(ts=ts, ts1=ts1, rho=rho, cost=cost, icosd=icosd, dmax=dmax.value, limps=limps.value)

    def set_mld_wind(self, mldketau):
        """imld = 1: new wind mixing energy mldketau, (maxj, maxi) = Fortran (maxi, maxj)."""
        a = np.ascontiguousarray(mldketau, dtype=np.float64)
        self._check(self.lib.gb_go_set_mld_wind(self.h, dptr(a)), "gb_go_set_mld_wind")

    def download_mld(self):
        """imld = 1: (mld, mldk) of the last step, each (maxj, maxi)."""
        mld = np.zeros((self.m.maxj, self.m.maxi))
        mldk = np.zeros((self.m.maxj, self.m.maxi), dtype=np.int32)
        self._check(self.lib.gb_go_download_mld(self.h, dptr(mld), iptr(mldk)), "gb_go_download_mld")
        return mld, mldk

    def inventory(self) -> np.ndarray:
        out = np.zeros(self.m.maxl)
        self._check(self.lib.gb_go_inventory(self.h, dptr(out)), "gb_go_inventory")
        return out

    def inventory_noalloc(self) -> np.ndarray:
        """The same inventory through gb_go_inventory_noalloc (static device scratch)."""
        out = np.zeros(self.m.maxl)
        self._check(self.lib.gb_go_inventory_noalloc(self.h, dptr(out)), "gb_go_inventory_noalloc")
        return out


def new_member_run(member, **kw) -> Goldstein:
    """Create a handle, upload the member's state and velocities."""
    g = Goldstein(member, **kw)
    g.upload_state()
    g.set_velocity()
    g.set_diag(member.cost, member.icosd)
    return g
