"""Batched ensembles of GOLDSTEIN grids over the gb_ens_* C-ABI.

Every member is an independent grid (its own dimensions, tracers, mask,
velocities and diffusivities).  All active members advance together, one
persistent FP32-flux launch per step; members can be added and retired between
steps (continuous batching).  There is no counterpart in the reference, which
runs a single grid serially; each member's arithmetic is the reference's
tracer step in the split-precision form (FP32 transfers, FP64 state).
"""
from __future__ import annotations

import ctypes as C
from typing import Optional

import numpy as np

from . import abi
from .abi import GbEnsTuning, GridRefs, dptr
from .goldstein import GoldsteinError, load_library


def host_empty(shape, dtype=np.float64) -> np.ndarray:
    """An uninitialised array in mapped page-locked host memory (gb_ens_host_alloc), freed with
    the array.  Ensemble.add_many reads ts and u that lie in such memory, and download_many
    writes ts, rho and cost there, through the device address inside the call's batched kernel
    (no copy call per array)."""
    import weakref
    lib = load_library()
    dt = np.dtype(dtype)
    n = int(np.prod(shape)) * dt.itemsize
    p = C.c_void_p()
    rc = lib.gb_ens_host_alloc(C.c_size_t(max(n, 1)), C.byref(p))
    if rc != 0:
        raise GoldsteinError(rc, "gb_ens_host_alloc")
    buf = (C.c_char * max(n, 1)).from_address(p.value)
    arr = np.frombuffer(buf, dtype=dt, count=int(np.prod(shape))).reshape(shape)
    weakref.finalize(buf, lib.gb_ens_host_free, C.c_void_p(p.value))
    return arr


def host_copy(a) -> np.ndarray:
    """host_empty filled with a copy of `a`."""
    out = host_empty(np.shape(a), np.asarray(a).dtype)
    out[...] = a
    return out


class Ensemble:
    def __init__(self, device: int = -1, hbm_budget_bytes: int = 0, *, tile_i: int = 0, tile_j: int = 0,
                 use_graph: bool = False, stream: Optional[int] = None, use_table: bool = True,
                 packing: Optional[int] = None, ctas_per_sm: Optional[int] = None, co_form: int = 0):
        """packing / ctas_per_sm: the batch's member packing (abi.GB_ENS_PACK_*) and cap on resident
        CTAs per SM; None = the autotuned values of the tuning table (else 0 and 0).  co_form: the
        convective adjustment's form (abi.GB_ENS_CO_*; 0: by the batch's size)."""
        self.lib = load_library()
        e = C.c_void_p()
        rc = self.lib.gb_ens_create(int(device), C.c_size_t(hbm_budget_bytes), C.byref(e))
        if rc != 0:
            raise GoldsteinError(rc, "gb_ens_create")
        self.e = e
        self.device = int(device)
        self.members = {}
        self.tile = (int(tile_i), int(tile_j))
        self.use_graph = bool(use_graph)
        self._current_tile = None
        from .autotune import batch_entry, load_table
        self.table = load_table() if use_table else {}
        tuned = batch_entry(self.table)
        self.packing = int(tuned[0] if packing is None else packing)
        self.ctas_per_sm = int(tuned[1] if ctas_per_sm is None else ctas_per_sm)
        self.co_form = int(co_form)
        self.set_tuning(tile_i=tile_i, tile_j=tile_j, use_graph=use_graph)
        if stream is not None:
            self._check(self.lib.gb_ens_set_stream(self.e, C.c_void_p(stream)), "gb_ens_set_stream")

    def _check(self, rc, what):
        if rc != 0:
            detail = self.lib.gb_ens_last_error(self.e).decode() if self.e else ""
            raise GoldsteinError(rc, what, detail)

    def set_tuning(self, tile_i=0, tile_j=0, ctas_per_sm=None, use_graph=False, packing=None):
        """gb_ens_set_tuning; ctas_per_sm / packing None: the ensemble's batch settings."""
        cps = self.ctas_per_sm if ctas_per_sm is None else int(ctas_per_sm)
        pk = self.packing if packing is None else int(packing)
        t = GbEnsTuning(int(tile_i), int(tile_j), cps, int(bool(use_graph)), pk, self.co_form)
        self._check(self.lib.gb_ens_set_tuning(self.e, C.byref(t)), "gb_ens_set_tuning")

    def close(self):
        if getattr(self, "e", None):
            self.lib.gb_ens_destroy(self.e)
            self.e = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    @staticmethod
    def member_bytes(member) -> int:
        lib = load_library()
        r = GridRefs(member)
        return int(lib.gb_ens_member_bytes(C.byref(r.dims), C.byref(r.params)))

    def _tile_for(self, member):
        """Tile shape: the one given at construction, else the autotuned one for this grid shape."""
        tile = self.tile
        if tile == (0, 0):
            from .autotune import lookup
            tile = lookup(self.table, member.maxi, member.maxj, member.maxk) or (0, 0)
        return tile

    def add(self, member, steps: Optional[int] = None, **kw) -> int:
        """Admit a member (its state ts is also the initial ts1); returns its id.
        Raises GoldsteinError(GB_GO_ENOMEM) when it does not fit the HBM budget."""
        tile = self._tile_for(member)
        if tile != self._current_tile:
            self.set_tuning(tile_i=tile[0], tile_j=tile[1], use_graph=self.use_graph)
            self._current_tile = tile
        return self._add_now(member, steps, **kw)

    def add_many(self, members, steps=None, **kw) -> list:
        """Admit several members in one call per tile shape (gb_ens_add_many: host preparation
        on up to 16 threads inside the library, one synchronisation).  The calls run on a worker
        thread in order, smallest group first, while this thread builds the next group's
        arguments (ctypes releases the GIL during a call).  All or nothing: when a call fails,
        the members this method admitted before it leave again.  `steps`: per member, its
        remaining-step count (set_remaining), or None.  Returns the ids in order."""
        from concurrent.futures import ThreadPoolExecutor

        from .abi import GbDims, GbGrid, GbParams
        members = list(members)
        ids = [None] * len(members)
        groups = {}
        for n, m in enumerate(members):
            groups.setdefault(self._tile_for(m), []).append(n)
        vp = C.c_void_p

        def arguments(idx):
            k = len(idx)
            refs = [GridRefs(members[n], precision=abi.GB_GO_FP32FLUX, **kw) for n in idx]
            tss = [np.ascontiguousarray(members[n].ts, dtype=np.float64) for n in idx]
            us = [np.ascontiguousarray(members[n].u, dtype=np.float64) for n in idx]
            return (refs, tss, us, (GbDims * k)(*[r.dims for r in refs]), (GbParams * k)(*[r.params for r in refs]),
                    (GbGrid * k)(*[r.grid for r in refs]), (vp * k)(*[abi.addr(a) for a in tss]),
                    (vp * k)(*[abi.addr(a) for a in us]))

        def call(tile, idx, args):
            if tile != self._current_tile:
                self.set_tuning(tile_i=tile[0], tile_j=tile[1], use_graph=self.use_graph)
                self._current_tile = tile
            out = (C.c_int32 * len(idx))()
            _, _, _, dims, params, grids, tsp, up = args
            rc = self.lib.gb_ens_add_many(self.e, len(idx), dims, params, grids, tsp, up, out)
            return rc, list(out)

        order = sorted(groups.items(), key=lambda g: len(g[1]))
        pending = None   # (indices, arguments kept alive, future) of the call in flight

        def collect():
            # the call in flight: its ids are recorded (admitted or not) before anything else
            nonlocal pending
            pidx, _, fut = pending
            pending = None
            rc, out = fut.result()
            if rc == 0:
                for n, mid in zip(pidx, out):
                    ids[n] = int(mid)
                    self.members[int(mid)] = members[n]
            self._check(rc, "gb_ens_add_many")

        try:
            with ThreadPoolExecutor(max_workers=1) as pool:
                try:
                    for tile, idx in order:
                        args = arguments(idx)
                        if pending is not None:
                            collect()
                        pending = (idx, args, pool.submit(call, tile, idx, args))
                    if pending is not None:
                        collect()
                finally:
                    if pending is not None:
                        try:
                            collect()
                        except Exception:
                            pass
        except BaseException:
            for mid in ids:
                if mid is not None:
                    self.remove(mid)
            raise
        if steps is not None:
            for mid, st in zip(ids, steps):
                if st is not None:
                    self.set_remaining(mid, int(st))
        return ids

    def _add_now(self, member, steps, **kw) -> int:
        r = GridRefs(member, precision=abi.GB_GO_FP32FLUX, **kw)
        ts = np.ascontiguousarray(member.ts, dtype=np.float64)
        u = np.ascontiguousarray(member.u, dtype=np.float64)
        mid = C.c_int32()
        self._check(self.lib.gb_ens_add(self.e, C.byref(r.dims), C.byref(r.params), C.byref(r.grid), dptr(ts),
                                        dptr(u), C.byref(mid)), "gb_ens_add")
        self.members[mid.value] = member
        if steps is not None:
            self.set_remaining(mid.value, steps)
        return mid.value

    def remove(self, mid: int):
        self._check(self.lib.gb_ens_remove(self.e, int(mid)), "gb_ens_remove")
        self.members.pop(mid, None)

    def step(self, nsteps: int = 1):
        self._check(self.lib.gb_ens_step(self.e, int(nsteps)), "gb_ens_step")

    def set_remaining(self, mid: int, steps: int):
        self._check(self.lib.gb_ens_set_remaining(self.e, int(mid), C.c_int64(int(steps))), "gb_ens_set_remaining")

    def remaining(self, mid: int) -> int:
        v = C.c_int64()
        self._check(self.lib.gb_ens_remaining(self.e, int(mid), C.byref(v)), "gb_ens_remaining")
        return int(v.value)

    def download(self, mid: int) -> dict:
        m = self.members[mid]
        ts = np.empty_like(m.ts)
        rho = np.empty_like(m.rho)
        cost = np.empty_like(m.cost)
        self._check(self.lib.gb_ens_download(self.e, int(mid), dptr(ts), dptr(rho), dptr(cost)), "gb_ens_download")
        return dict(ts=ts, rho=rho, cost=cost)

    def download_many(self, mids, out=None) -> list:
        """download() of several members in one call (gb_ens_download_many: one kernel for all,
        copies queued behind the steps, one synchronisation).  `out`: one dict of ts, rho and
        cost arrays per member to write into (e.g. pinned host memory, which the copies reach
        without staging); new arrays otherwise."""
        mids = list(mids)
        outs = []
        for n, mid in enumerate(mids):
            m = self.members[mid]
            if out is not None:
                o = out[n]
                for key, ref in (("ts", m.ts), ("rho", m.rho), ("cost", m.cost)):
                    a = o[key]
                    if a.shape != ref.shape or a.dtype != np.float64 or not a.flags.c_contiguous:
                        raise ValueError("download_many: output arrays must match the member's shapes (float64, C order)")
                outs.append(o)
            else:
                outs.append(dict(ts=np.empty_like(m.ts), rho=np.empty_like(m.rho), cost=np.empty_like(m.cost)))
        n = len(mids)
        if n == 0:
            return outs
        dp = C.POINTER(C.c_double)
        ids = (C.c_int32 * n)(*mids)
        arr = {key: (dp * n)(*[dptr(o[key]) for o in outs]) for key in ("ts", "rho", "cost")}
        self._check(self.lib.gb_ens_download_many(self.e, n, ids, arr["ts"], arr["rho"], arr["cost"]),
                    "gb_ens_download_many")
        return outs

    def set_mld_wind(self, mid: int, mldketau):
        """imld = 1 members: the wind mixing energy per column ((maxj, maxi) array) from the next
        step on (gb_ens_set_mld_wind)."""
        a = np.ascontiguousarray(mldketau, dtype=np.float64)
        self._check(self.lib.gb_ens_set_mld_wind(self.e, int(mid), dptr(a)), "gb_ens_set_mld_wind")

    def download_mld(self, mid: int):
        """imld = 1 members: (mld, mldk), the mixed-layer depth and level of every column as
        (maxj, maxi) arrays (gb_ens_download_mld)."""
        m = self.members[mid]
        mld = np.zeros((m.maxj, m.maxi))
        mldk = np.zeros((m.maxj, m.maxi), dtype=np.int32)
        self._check(self.lib.gb_ens_download_mld(self.e, int(mid), dptr(mld), abi.iptr(mldk)), "gb_ens_download_mld")
        return mld, mldk

    def inventory(self, mid: int) -> np.ndarray:
        out = np.zeros(self.members[mid].maxl)
        self._check(self.lib.gb_ens_inventory(self.e, int(mid), dptr(out)), "gb_ens_inventory")
        return out

    def status(self, mid: int) -> int:
        v = C.c_int32()
        self._check(self.lib.gb_ens_status(self.e, int(mid), C.byref(v)), "gb_ens_status")
        return int(v.value)

    def sync(self):
        self._check(self.lib.gb_ens_sync(self.e), "gb_ens_sync")

    def count(self):
        a = C.c_int32()
        b = C.c_size_t()
        self._check(self.lib.gb_ens_count(self.e, C.byref(a), C.byref(b)), "gb_ens_count")
        return int(a.value), int(b.value)
