"""ctypes mirror of include/gb_goldstein.h (structs, constants) and helpers that
fill them from a :class:`cgenie_gb300.grid.Member`.

The structs carry what the reference's ``tstepo`` reads from module state
(src/goldstein/goldstein_lib.f90:6-180): dimensions, namelist switches and
grid metrics.  Pointers in ``GbGrid`` reference numpy arrays that the caller
must keep alive for the duration of the C call (``GridRefs`` does that).
"""
from __future__ import annotations

import ctypes as C

import numpy as np

GB_GO_OK = 0
GB_GO_EINVAL = -1
GB_GO_EUNSUPPORTED = -2
GB_GO_ECUDA = -3
GB_GO_ENOMEM = -4
GB_GO_ENOTREADY = -5
GB_GO_EDEVICE = -6
GB_GO_ERANGE = -7
GB_GO_ENONFINITE = -8

GB_GO_FP64 = 0
GB_GO_FP32FLUX = 1
GB_GO_MAX_K = 64
GB_GO_MAX_L = 128

ERRNAMES = {
    GB_GO_EINVAL: "EINVAL", GB_GO_EUNSUPPORTED: "EUNSUPPORTED", GB_GO_ECUDA: "ECUDA",
    GB_GO_ENOMEM: "ENOMEM", GB_GO_ENOTREADY: "ENOTREADY", GB_GO_EDEVICE: "EDEVICE",
    GB_GO_ERANGE: "ERANGE", GB_GO_ENONFINITE: "ENONFINITE",
}

_dp = C.POINTER(C.c_double)
_ip = C.POINTER(C.c_int32)


class GbDims(C.Structure):
    _fields_ = [("maxi", C.c_int32), ("maxj", C.c_int32), ("maxk", C.c_int32), ("maxl", C.c_int32)]


class GbParams(C.Structure):
    _fields_ = [
        ("diff", C.c_double * 2),
        ("ec", C.c_double * 5),
        ("ediff0", C.c_double),
        ("ediffpow2", C.c_double),
        ("dsc", C.c_double),
        ("ieos", C.c_int32),
        ("iediff", C.c_int32),
        ("ediffpow2i", C.c_int32),
        ("iconv", C.c_int32),
        ("imld", C.c_int32),
        ("diso", C.c_int32),
        ("precision", C.c_int32),
        ("reserved", C.c_int32),
        ("mldpebuoycoeff", C.c_double),
    ]


_vp = C.c_void_p   # array addresses (const double * / const int32_t * in C); set from numpy addresses


class GbGrid(C.Structure):
    _fields_ = [
        ("rc", _vp), ("rc2", _vp), ("cv", _vp),
        ("cv2", _vp), ("dsv", _vp), ("rdsv", _vp),
        ("ds", _vp), ("rds", _vp),
        ("dz", _vp), ("dza", _vp), ("rdz", _vp), ("rdza", _vp), ("zro", _vp), ("dt", _vp),
        ("zw", _vp),
        ("ssmax", _vp),
        ("ediff1", _vp),
        ("diffmax", _vp),
        ("k1", _vp),
        ("dphi", C.c_double), ("rdphi", C.c_double),
        ("mlddec", _vp), ("mlddecd", _vp), ("mldketau", _vp),
    ]


class GbBgDims(C.Structure):
    """gb_bg_dims (include/gb_biogem.h)."""
    _fields_ = [("n_i", C.c_int32), ("n_j", C.c_int32), ("n_k", C.c_int32), ("n_l_ocn", C.c_int32),
                ("n_l_sed", C.c_int32), ("pad", C.c_int32)]


class GbBgParams(C.Structure):
    """gb_bg_params: tstoocn_offset(1:2) and ctrl_force_GOLDSTEInTS."""
    _fields_ = [("ts_offset", C.c_double * 2), ("force_ts", C.c_int32), ("pad", C.c_int32)]


class GbRsCalendar(C.Structure):
    """gb_rs_calendar: iyear_rest, imonth_rest, ioffset_rest, istep_ocn and day_rest."""
    _fields_ = [("iyear", C.c_int32), ("imonth", C.c_int32), ("ioffset", C.c_int32), ("istep", C.c_int32),
                ("day", C.c_double)]


GB_EA_EMBM = 0
GB_EA_SEAICE = 1
GB_EA_SEAICE_EXPLICIT = 2
GB_EA_MAX_CELLS = 32768


class GbEaDims(C.Structure):
    """gb_ea_dims (include/gb_embm.h)."""
    _fields_ = [("maxi", C.c_int32), ("maxj", C.c_int32)]


class GbEaParams(C.Structure):
    """gb_ea_params: the scalars of tstipa (EMBM) or tstipsic (sea ice)."""
    _fields_ = [("kind", C.c_int32), ("maxk", C.c_int32), ("dt", C.c_double), ("dphi", C.c_double),
                ("rdphi", C.c_double), ("betaz", C.c_double * 2), ("betam", C.c_double * 2),
                ("diffmod0", C.c_double), ("ppmin", C.c_double), ("ppmax", C.c_double),
                ("diffsic", C.c_double), ("tsc", C.c_double), ("sica_thresh", C.c_double),
                ("sich_thresh", C.c_double)]


class GbEaSeaicePost(C.Structure):
    """gb_ea_seaice_post: the constants of step_seaice's post-processing."""
    _fields_ = [("rhoio", C.c_double), ("rhoice", C.c_double), ("hlf", C.c_double), ("hmin", C.c_double),
                ("rdtdim", C.c_double), ("m2mm", C.c_double)]


class GbEaGrid(C.Structure):
    """gb_ea_grid: j metrics with their Fortran bounds, diffa (EMBM) or k1 (sea ice)."""
    _fields_ = [("rc", _dp), ("cv", _dp), ("dsv", _dp), ("rdsv", _dp), ("rds", _dp), ("diffa", _dp),
                ("k1", _ip)]


class GbEnsTuning(C.Structure):
    _fields_ = [("tile_i", C.c_int32), ("tile_j", C.c_int32), ("ctas_per_sm", C.c_int32),
                ("use_graph", C.c_int32), ("packing", C.c_int32), ("co_form", C.c_int32)]


GB_ENS_PACK_MEMBERS, GB_ENS_PACK_ITEMS, GB_ENS_PACK_ROUND_ROBIN = 0, 1, 2
GB_ENS_CO_AUTO, GB_ENS_CO_WARP, GB_ENS_CO_TWO_PHASE = 0, 1, 2
GB_ENS_CO_TWO_PHASE_MIN = 100000


def addr(a: np.ndarray) -> int:
    """Address of a contiguous array's first element (ctypes' buffer view for writable arrays,
    a third of the cost of __array_interface__)."""
    try:
        return C.addressof(C.c_char.from_buffer(a))
    except (TypeError, ValueError):
        return a.__array_interface__["data"][0]


def dptr(a: np.ndarray):
    """Pointer to a contiguous float64 numpy array (None -> NULL)."""
    if a is None:
        return None
    assert a.dtype == np.float64 and a.flags["C_CONTIGUOUS"], (a.dtype, a.flags)
    return a.ctypes.data_as(_dp)


def iptr(a: np.ndarray):
    if a is None:
        return None
    assert a.dtype == np.int32 and a.flags["C_CONTIGUOUS"], (a.dtype, a.flags)
    return a.ctypes.data_as(_ip)


class GridRefs:
    """Owns contiguous copies of a member's metric arrays and the ctypes structs
    that point at them."""

    _F64 = ("rc", "rc2", "cv", "cv2", "dsv", "rdsv", "ds", "rds", "dz", "dza", "rdz", "rdza", "zro", "dt", "zw",
            "ssmax", "ediff1", "diffmax")
    _MLD = ("mlddec", "mlddecd", "mldketau")

    def __init__(self, m, *, diso=None, ieos=None, iconv=None, iediff=None, imld=None, precision=GB_GO_FP64):
        cfg = m.cfg
        f64 = np.float64
        asc = np.ascontiguousarray
        arrays = {name: asc(getattr(m, name), dtype=f64) for name in self._F64}
        arrays["k1"] = asc(m.k1, dtype=np.int32)
        for name in self._MLD:
            v = getattr(m, name, None)
            arrays[name] = None if v is None else asc(v, dtype=f64)
        self.arrays = arrays
        self.dims = GbDims(m.maxi, m.maxj, m.maxk, m.maxl)
        diff, ec = m.diff, m.ec
        self.params = GbParams(
            diff=(C.c_double * 2)(float(diff[0]), float(diff[1])), ec=(C.c_double * 5)(*[float(x) for x in ec[:5]]),
            ediff0=float(m.ediff0), ediffpow2=float(m.ediffpow2), dsc=5.0e3,
            ieos=int(cfg.ieos if ieos is None else ieos), iediff=int(cfg.iediff if iediff is None else iediff),
            ediffpow2i=int(m.ediffpow2i), iconv=int(cfg.iconv if iconv is None else iconv),
            imld=int(getattr(cfg, "imld", 0) if imld is None else imld),
            diso=int(bool(cfg.diso if diso is None else diso)), precision=int(precision), reserved=0,
            mldpebuoycoeff=float(getattr(cfg, "mldpebuoycoeff", 0.15)))
        ptr = {name: (None if a is None else addr(a)) for name, a in arrays.items()}   # contiguous, or None
        self.grid = GbGrid(*[ptr[name] for name in self._F64], ptr["k1"], float(m.dphi), float(m.rdphi),
                           *[ptr[name] for name in self._MLD])
