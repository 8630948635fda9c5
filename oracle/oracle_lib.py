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

from cgenie_gb300.abi import GbDims, GbParams, GbGrid, GridRefs, dptr, iptr

HERE = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(HERE, "_build", "libgb_oracle.so")

_lib = None


def build(force: bool = False) -> str:
    """Compile the oracle (make -C oracle)."""
    src = os.path.join(HERE, "goldstein_oracle.c")
    if force or not os.path.exists(LIB_PATH) or os.path.getmtime(LIB_PATH) < os.path.getmtime(src):
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
