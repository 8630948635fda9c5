"""ORACLE -- test infrastructure only.  ctypes wrapper of oracle/_build/libgb_oracle.so
(the C restatement of src/goldstein/goldstein.f90:2280-2842,3048-3082).

Only tests/, __graft_entry__.smoke() and bench.py's CPU-baseline leg import
this module.
"""
from __future__ import annotations

import ctypes as C
import os
import subprocess

import numpy as np

from cgenie_gb300.abi import (GbBgDims, GbBgParams, GbDims, GbEaDims, GbEaGrid, GbEaParams, GbGrid, GbParams,
                              GridRefs, dptr, iptr)

HERE = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(HERE, "_build", "libgb_oracle.so")

_lib = None


def build(force: bool = False) -> str:
    """Compile the oracle (make -C oracle)."""
    srcs = [os.path.join(HERE, f) for f in ("goldstein_oracle.c", "biogem_oracle.c", "surface_oracle.c",
                                             "momentum_oracle.c", "timeseries_oracle.c")]
    if force or not os.path.exists(LIB_PATH) or os.path.getmtime(LIB_PATH) < max(os.path.getmtime(f) for f in srcs):
        subprocess.run(["make", "-s", "-C", HERE], check=True)
    return LIB_PATH


def lib():
    global _lib
    if _lib is None:
        build()
        L = C.CDLL(LIB_PATH)
        P = C.POINTER
        L.gbo_tstepo.argtypes = [P(GbDims), P(GbParams), P(GbGrid), P(C.c_double), P(C.c_double),
                                 P(C.c_double), P(C.c_double), P(C.c_double), P(C.c_int32),
                                 P(C.c_double), P(C.c_int32), C.c_int32, C.c_int32]
        L.gbo_tstepo.restype = C.c_int
        L.gbo_tstepo_mld.argtypes = L.gbo_tstepo.argtypes + [P(C.c_double), P(C.c_int32)]
        L.gbo_tstepo_mld.restype = C.c_int
        L.gbo_tstepo_flux.argtypes = [P(GbDims), P(GbParams), P(GbGrid), P(C.c_double), P(C.c_double),
                                      P(C.c_double), P(C.c_double), P(C.c_double), P(C.c_int32)]
        L.gbo_tstepo_flux.restype = C.c_int
        L.gbo_co.argtypes = [P(GbDims), P(GbParams), P(GbGrid), P(C.c_double), P(C.c_double),
                             P(C.c_double), P(C.c_int32)]
        L.gbo_co.restype = C.c_int
        L.gbo_eos.argtypes = [P(C.c_double), C.c_double, C.c_double, C.c_double, C.c_int32]
        L.gbo_eos.restype = C.c_double
        L.gbo_eosd.argtypes = [P(C.c_double), C.c_double, C.c_double, C.c_double, C.c_double, C.c_double,
                               C.c_double, C.c_int32, P(C.c_double), P(C.c_double)]
        L.gbo_eosd.restype = None
        L.gbo_inventory.argtypes = [P(GbDims), P(GbGrid), P(C.c_double), P(C.c_double)]
        L.gbo_inventory.restype = C.c_int
        dp = P(C.c_double)
        L.gbo_bg_tracercoupling.argtypes = [P(GbBgDims), P(GbBgParams), P(C.c_int32), dp, dp, dp, dp, dp, dp,
                                            dp, dp, dp]
        L.gbo_bg_tracercoupling.restype = C.c_int
        L.gbo_bg_columns.argtypes = [P(GbBgDims), P(C.c_int32)]
        L.gbo_bg_columns.restype = C.c_int
        L.gbo_ea_step.argtypes = [P(GbEaDims), P(GbEaParams), P(GbEaGrid), dp, dp, dp, dp, dp, C.c_int]
        L.gbo_ea_step.restype = C.c_int
        L.gbo_mo_init.argtypes = [C.c_void_p, C.c_void_p, C.c_void_p]
        L.gbo_mo_init.restype = C.c_void_p
        L.gbo_mo_step.argtypes = [C.c_void_p, dp, dp, dp, dp]
        L.gbo_mo_step.restype = C.c_int
        L.gbo_mo_get.argtypes = [C.c_void_p, dp, dp, dp, dp, dp, dp]
        L.gbo_mo_get.restype = None
        L.gbo_mo_matrix.argtypes = [C.c_void_p, dp]
        L.gbo_mo_matrix.restype = None
        L.gbo_mo_get_islands.argtypes = [C.c_void_p, dp, dp, dp]
        L.gbo_mo_get_islands.restype = None
        L.gbo_mo_set_velocity.argtypes = [C.c_void_p, dp, dp]
        L.gbo_mo_set_velocity.restype = None
        L.gbo_mo_free.argtypes = [C.c_void_p]
        L.gbo_mo_free.restype = None
        from cgenie_gb300.timeseries import GbTsBasins
        L.gbo_diag2.argtypes = [P(GbDims), P(GbGrid), P(GbTsBasins), dp, dp, dp, dp, dp, dp]
        L.gbo_diag2.restype = C.c_int
        L.gbo_diagopsi.argtypes = [P(GbDims), P(GbGrid), P(GbTsBasins), dp, dp, dp, dp, dp, P(C.c_int32)]
        L.gbo_diagopsi.restype = C.c_int
        _lib = L
    return _lib


class OracleState:
    """A member's state advanced by the C oracle (in place on Fortran-layout arrays)."""

    def __init__(self, m, refs: GridRefs | None = None, **kw):
        self.m = m
        self.refs = refs or GridRefs(m, **kw)
        self.ts = m.ts.copy()
        self.ts1 = m.ts1.copy()
        self.rho = m.rho.copy()
        self.u = np.ascontiguousarray(m.u)
        self.cost = m.cost.copy()
        self.icosd = m.icosd.copy()
        self.dmax = C.c_double(0.0)
        self.limps = C.c_int32(0)
        mld = getattr(m, "mld", None)
        self.mld = np.zeros((m.maxj, m.maxi)) if mld is None else mld.copy()
        mldk = getattr(m, "mldk", None)
        self.mldk = np.zeros((m.maxj, m.maxi), dtype=np.int32) if mldk is None else mldk.copy()

    def step(self, nsteps: int = 1, faithful: bool = False) -> None:
        r = self.refs
        rc = lib().gbo_tstepo_mld(C.byref(r.dims), C.byref(r.params), C.byref(r.grid), dptr(self.ts),
                                  dptr(self.ts1), dptr(self.rho), dptr(self.u), dptr(self.cost),
                                  iptr(self.icosd), C.byref(self.dmax), C.byref(self.limps),
                                  int(nsteps), int(bool(faithful)), dptr(self.mld), iptr(self.mldk))
        if rc != 0:
            raise RuntimeError(f"oracle gbo_tstepo failed: {rc}")

    def inventory(self) -> np.ndarray:
        out = np.zeros(self.m.maxl)
        r = self.refs
        rc = lib().gbo_inventory(C.byref(r.dims), C.byref(r.grid), dptr(self.ts), dptr(out))
        if rc != 0:
            raise RuntimeError(f"oracle gbo_inventory failed: {rc}")
        return out


def run(m, nsteps: int, **kw) -> OracleState:
    s = OracleState(m, **kw)
    s.step(nsteps)
    return s


def go_ts_interior(ts: np.ndarray) -> np.ndarray:
    """go_ts (n_l_ocn, n_i, n_j, n_k) from a halo'd ts array ([k, j, i, l] C order)."""
    m_k = ts.shape[0] - 2
    return np.ascontiguousarray(ts[1:m_k + 1, 1:-1, 1:-1, :])


def bg_tracercoupling(m, st, go_ts: np.ndarray, *, force_ts: bool = False, ts_offset=(273.15, 34.9)):
    """The C restatement of biogem_tracercoupling on go_ts ([k, j, i, l] C order, interior only)
    and a BiogemState `st` (updated in place).  Returns (go_ts, go_ts1)."""
    L, Ls = m.maxl, st.vbio_part.shape[-1]
    d = GbBgDims(m.maxi, m.maxj, m.maxk, L, Ls, 0)
    p = GbBgParams((C.c_double * 2)(*ts_offset), int(bool(force_ts)), 0)
    k1 = np.ascontiguousarray(m.k1[1:m.maxj + 1, 1:m.maxi + 1], dtype=np.int32)
    ts = np.ascontiguousarray(go_ts, dtype=np.float64).copy()
    ts1 = np.zeros_like(ts)
    for name in ("vocn", "mass", "volume", "rmass", "vbio_part", "vdocn", "vdbio_part"):
        setattr(st, name, np.ascontiguousarray(getattr(st, name), dtype=np.float64))
    nul = C.POINTER(C.c_double)()
    rc = lib().gbo_bg_tracercoupling(C.byref(d), C.byref(p), iptr(k1), dptr(ts), dptr(ts1), dptr(st.vocn),
                                     dptr(st.mass), dptr(st.volume), dptr(st.rmass), dptr(st.vdocn),
                                     dptr(st.vbio_part) if Ls else nul, dptr(st.vdbio_part) if Ls else nul)
    if rc != 0:
        raise RuntimeError(f"oracle gbo_bg_tracercoupling failed: {rc}")
    return ts, ts1


def after_coupling(state: "OracleState", go_ts: np.ndarray, go_ts1: np.ndarray) -> None:
    """step_goldstein's copy-in and boundary conditions after a coupling
    (src/goldstein/goldstein.f90:176-187): ts and ts1 interiors from go_ts / go_ts1, then
    ts1's periodic i-halo from ts."""
    m = state.m
    mk = m.maxk
    state.ts[1:mk + 1, 1:-1, 1:-1, :] = go_ts
    state.ts1[1:mk + 1, 1:-1, 1:-1, :] = go_ts1
    for j in range(1, m.maxj + 1):
        for k in range(int(m.k1[j, 0]), mk + 1):
            state.ts1[k, j, 0, :] = state.ts[k, j, m.maxi, :]
        for k in range(int(m.k1[j, m.maxi + 1]), mk + 1):
            state.ts1[k, j, m.maxi + 1, :] = state.ts[k, j, 1, :]


def surface_step(case, nsteps: int = 1):
    """The C restatement of tstipa / tstipsic on a cgenie_gb300.surface.SurfaceCase (its tq,
    tq1 are updated in place)."""
    d = GbEaDims(case.maxi, case.maxj)
    p = case.params()
    g = case.grid()
    case.tq = np.ascontiguousarray(case.tq, dtype=np.float64)
    case.tq1 = np.ascontiguousarray(case.tq1, dtype=np.float64)
    src = np.ascontiguousarray(case.source, dtype=np.float64)
    vel = np.ascontiguousarray(case.vel, dtype=np.float64)
    pp = None if case.pptn is None else np.ascontiguousarray(case.pptn, dtype=np.float64)
    rc = lib().gbo_ea_step(C.byref(d), C.byref(p), C.byref(g), dptr(case.tq), dptr(case.tq1), dptr(src), dptr(vel),
                           dptr(pp), int(nsteps))
    if rc != 0:
        raise RuntimeError(f"oracle gbo_ea_step failed: {rc}")


class OracleMomentum:
    """The C restatement of the momentum step (oracle/momentum_oracle.c) on a
    cgenie_gb300.momentum.MomentumCase."""

    def __init__(self, case):
        self.case = case
        self._d, self._p, self._g = case.dims(), case.params(), case.grid()
        self.s = lib().gbo_mo_init(C.byref(self._d), C.byref(self._p), C.byref(self._g))
        if not self.s:
            raise RuntimeError("oracle gbo_mo_init failed")

    def close(self):
        if self.s:
            lib().gbo_mo_free(self.s)
            self.s = None

    def __del__(self):
        self.close()

    def step(self, rho, tau=None, dztau=None, dztav=None):
        c = self.case
        arrs = [np.ascontiguousarray(x, dtype=np.float64) for x in
                (c.tau if tau is None else tau, c.dztau if dztau is None else dztau,
                 c.dztav if dztav is None else dztav, rho)]
        lib().gbo_mo_step(self.s, *[dptr(a) for a in arrs])

    def state(self):
        c = self.case
        nu = (c.maxk, c.maxj + 1, c.maxi + 1, 3)
        u, u1 = np.zeros(nu), np.zeros(nu)
        ub = np.zeros((c.maxj + 1, c.maxi + 2, 2))
        psi = np.zeros((c.maxj + 1, c.maxi + 1))
        lib().gbo_mo_get(self.s, dptr(u), dptr(u1), dptr(ub), dptr(psi), None, None)
        return dict(u=u, u1=u1, ub=ub, psi=psi)

    def matrix(self):
        nm = self.case.maxi * (self.case.maxj + 1)
        A = np.zeros((nm, nm))
        lib().gbo_mo_matrix(self.s, dptr(A))
        return A

    def islands(self):
        c = self.case
        psisl = np.zeros((c.isles, c.maxj + 1, c.maxi + 1))
        ubisl = np.zeros((c.isles, c.maxj + 1, c.maxi + 2, 2))
        erisl = np.zeros((c.isles + 1, c.isles))
        lib().gbo_mo_get_islands(self.s, dptr(psisl), dptr(ubisl), dptr(erisl))
        return psisl, ubisl, erisl


def timeseries(m, ts, rho, u, basins):
    """diag2 and diagopsi of the oracle (oracle/timeseries_oracle.c) on Fortran-layout arrays."""
    r = GridRefs(m)
    cb = basins.c()
    sums = np.zeros(8 * m.maxl)
    avn, avs = C.c_double(), C.c_double()
    shape = (m.maxk + 1, m.maxj + 1)
    ops = [np.zeros(shape) for _ in range(3)]
    ext = np.zeros(4)
    iposa = np.zeros(2, np.int32)
    a = [np.ascontiguousarray(x, dtype=np.float64) for x in (ts, rho, u)]
    lib().gbo_diag2(C.byref(r.dims), C.byref(r.grid), C.byref(cb), dptr(a[0]), dptr(a[1]), dptr(a[2]), dptr(sums),
                    C.byref(avn), C.byref(avs))
    lib().gbo_diagopsi(C.byref(r.dims), C.byref(r.grid), C.byref(cb), dptr(a[2]), *[dptr(o) for o in ops], dptr(ext),
                       iptr(iposa))
    return dict(sums=sums, avn=avn.value, avs=avs.value, ext=ext, iposa=iposa, opsi=ops[0], opsip=ops[1], opsia=ops[2])

