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


class Ensemble:
    def __init__(self, device: int = -1, hbm_budget_bytes: int = 0, *, tile_i: int = 0, tile_j: int = 0,
                 use_graph: bool = False, stream: Optional[int] = None, use_table: bool = True):
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
        from .autotune import load_table
        self.table = load_table() if use_table else {}
        self.set_tuning(tile_i=tile_i, tile_j=tile_j, use_graph=use_graph)
        if stream is not None:
            self._check(self.lib.gb_ens_set_stream(self.e, C.c_void_p(stream)), "gb_ens_set_stream")

    def _check(self, rc, what):
        if rc != 0:
            detail = self.lib.gb_ens_last_error(self.e).decode() if self.e else ""
            raise GoldsteinError(rc, what, detail)

    def set_tuning(self, tile_i=0, tile_j=0, ctas_per_sm=0, use_graph=False):
        t = GbEnsTuning(int(tile_i), int(tile_j), int(ctas_per_sm), int(bool(use_graph)))
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

    def add_many(self, members, threads: Optional[int] = None, **kw) -> list:
        """Admit several members; their host-side preparation (patch plan, coefficients,
        scales) runs in parallel threads, as gb_ens_add allows.  Returns the ids in order."""
        import os
        from concurrent.futures import ThreadPoolExecutor
        members = list(members)
        ids = [None] * len(members)
        groups = {}
        for n, m in enumerate(members):
            groups.setdefault(self._tile_for(m), []).append(n)
        workers = threads or min(16, os.cpu_count() or 1)
        with ThreadPoolExecutor(max_workers=workers) as ex:
            for tile, idx in groups.items():
                if tile != self._current_tile:
                    self.set_tuning(tile_i=tile[0], tile_j=tile[1], use_graph=self.use_graph)
                    self._current_tile = tile
                for n, mid in zip(idx, ex.map(lambda n: self._add_now(members[n], None, **kw), idx)):
                    ids[n] = mid
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

    def download_many(self, mids, threads: int = 8, out=None) -> list:
        """download() of several members from host threads, each with its own CUDA stream
        (gb_ens_download_stream), so that the device-to-host copies overlap.  `out`: one dict
        of ts, rho and cost arrays per member to write into (e.g. pinned host memory, which
        the copies reach without staging); new arrays otherwise."""
        import queue
        from concurrent.futures import ThreadPoolExecutor
        import torch
        mids = list(mids)
        dev = torch.device("cuda", self.device if self.device >= 0 else torch.cuda.current_device())
        free = queue.Queue()
        for _ in range(threads):
            free.put(torch.cuda.Stream(device=dev))
        dst = dict(zip(mids, out)) if out is not None else {}

        def one(mid):
            m = self.members[mid]
            if mid in dst:
                ts, rho, cost = dst[mid]["ts"], dst[mid]["rho"], dst[mid]["cost"]
                for a, ref in ((ts, m.ts), (rho, m.rho), (cost, m.cost)):
                    if a.shape != ref.shape or a.dtype != np.float64 or not a.flags.c_contiguous:
                        raise ValueError("download_many: output arrays must match the member's shapes (float64, C order)")
            else:
                ts, rho, cost = np.empty_like(m.ts), np.empty_like(m.rho), np.empty_like(m.cost)
            st = free.get()
            try:
                self._check(self.lib.gb_ens_download_stream(self.e, int(mid), C.c_void_p(st.cuda_stream), dptr(ts),
                                                            dptr(rho), dptr(cost)), "gb_ens_download_stream")
            finally:
                free.put(st)
            return dict(ts=ts, rho=rho, cost=cost)
        with ThreadPoolExecutor(max_workers=threads) as ex:
            return list(ex.map(one, mids))

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
