"""Continuous-batching service for ensemble-member runs.

A request asks for `steps` tracer steps of one member (grid 18x18x16, 36x36x16
or 36x36x32, 2-24 tracers, seeded mask, velocities and diffusivities).  The
loop admits arrived requests into the running ensemble while the HBM budget
allows (gb_ens_add reports GB_GO_ENOMEM otherwise and the request waits),
advances every admitted member together in chunks of steps, and retires
members whose step count is reached (download, then free).  Latency of a run
is completion minus arrival; throughput is tracer cell-updates per second of
wall time.  Each member's arithmetic does not depend on which other members
share the batch, so a result is the same alone and in the mix.
"""
from __future__ import annotations

import collections
import dataclasses
import math
import time
from typing import Callable, Optional

import numpy as np

from . import abi, grid
from .ensemble import Ensemble
from .goldstein import GoldsteinError

SHAPES = [(18, 18, 16), (36, 36, 16), (36, 36, 32)]


@dataclasses.dataclass
class Request:
    rid: int
    shape: tuple
    maxl: int
    variant: int
    diff_h: float
    diff_v: float
    steps: int
    arrival: float
    admitted: float = math.nan
    finished: float = math.nan
    cell_updates: int = 0
    member_id: int = -1
    steps_left: int = 0
    result: Optional[dict] = None


class MemberFactory:
    """Seeded members, built once per (shape, variant) with 24 tracers and then
    specialised per request (tracer count, diffusivities) without regenerating
    the mask and velocity field."""

    def __init__(self, variants: int = 4, seed: int = 2024, lmax: int = 24):
        self.base = {}
        self.variants = variants
        self.seed = seed
        self.lmax = lmax

    def base_member(self, shape, variant):
        key = (shape, variant)
        if key not in self.base:
            mi, mj, mk = shape
            cfg = grid.MemberConfig(maxi=mi, maxj=mj, maxk=mk, maxl=self.lmax, seed=self.seed + 97 * variant + mk,
                                    tracer_kind="bgc")
            self.base[key] = grid.make_member(cfg)
        return self.base[key]

    def member(self, req: Request):
        b = self.base_member(req.shape, req.variant)
        m = dataclasses.replace(b)
        m.maxl = req.maxl
        m.ts = np.ascontiguousarray(b.ts[..., :req.maxl])
        m.ts1 = m.ts
        m.diff = np.array([req.diff_h / (grid.RSC * grid.USC), req.diff_v * grid.RSC / (grid.USC * grid.DSC ** 2)])
        m.cfg = dataclasses.replace(b.cfg, maxl=req.maxl, diff_h=req.diff_h, diff_v=req.diff_v)
        return m


def poisson_requests(n: int, rate: float = 50.0, seed: int = 7, smin: int = 200, smax: int = 5000,
                     lmin: int = 2, lmax: int = 24, variants: int = 4):
    rng = np.random.default_rng(seed)
    t = 0.0
    out = []
    for r in range(n):
        t += rng.exponential(1.0 / rate)
        out.append(Request(
            rid=r, shape=SHAPES[int(rng.integers(0, 3))], maxl=int(rng.integers(lmin, lmax + 1)),
            variant=int(rng.integers(0, variants)),
            diff_h=float(math.exp(rng.uniform(math.log(500.0), math.log(5000.0)))),
            diff_v=float(math.exp(rng.uniform(math.log(1e-6), math.log(1e-4)))),
            steps=int(rng.integers(smin, smax + 1)), arrival=t))
    return out


class Server:
    """The serving loop over one Ensemble on its own CUDA stream.  Each round launches the next
    chunk of batched steps (asynchronously), admits the requests that arrived meanwhile while the
    chunk runs (their host preparation overlaps the GPU work; their device set-up is queued
    behind the chunk, so they join at the next step boundary), synchronises, and retires the
    members whose step count is reached.  GPU busy time is the chunks' CUDA-event time."""

    def __init__(self, hbm_budget_bytes: int = 0, chunk: int = 25, device: int = -1, keep_results: bool = False,
                 use_graph: bool = False, factory: Optional[MemberFactory] = None):
        import torch
        dev = torch.device("cuda", device if device >= 0 else torch.cuda.current_device())
        self.stream = torch.cuda.Stream(device=dev)
        self.ens = Ensemble(device=device, hbm_budget_bytes=hbm_budget_bytes, use_graph=use_graph,
                            stream=self.stream.cuda_stream)
        self.chunk = chunk
        self.keep = keep_results
        self.factory = factory or MemberFactory()
        self.wet = {}

    def close(self):
        self.ens.close()

    def _wet(self, m):
        key = (m.maxi, m.maxj, m.maxk, id(m.k1))
        if key not in self.wet:
            self.wet[key] = m.wet_cells
        return self.wet[key]

    def _admit(self, waiting, active, stamp):
        """Admit waiting requests in arrival order while the HBM budget allows: all of them in
        one batched call, else (the budget is short) one at a time until one does not fit."""
        if not waiting:
            return
        reqs = list(waiting)
        ms = [self.factory.member(r) for r in reqs]
        try:
            ids = self.ens.add_many(ms, steps=[r.steps for r in reqs])
        except GoldsteinError as e:
            if e.code != abi.GB_GO_ENOMEM:
                raise
            ids = []
            for r, m in zip(reqs, ms):
                try:
                    ids.append(self.ens.add(m, steps=r.steps))
                except GoldsteinError as e2:
                    if e2.code == abi.GB_GO_ENOMEM:
                        break
                    raise
        now = stamp()
        for req, m, mid in zip(reqs, ms, ids):
            waiting.popleft()
            req.member_id = mid
            req.admitted = now
            req.cell_updates = self._wet(m) * req.maxl * req.steps
            req.steps_left = req.steps     # the library's remaining-step count, kept on the host
            active[mid] = req

    def run(self, requests, clock: Callable[[], float] = time.perf_counter, time_scale: float = 1.0):
        """Serve `requests` (arrival times in seconds from the start).  Returns stats."""
        import torch
        pending = collections.deque(sorted(requests, key=lambda r: r.arrival))
        waiting = collections.deque()
        active = {}
        done = []
        ens = self.ens
        t0 = clock()
        stamp = lambda: (clock() - t0) * time_scale   # noqa: E731
        total_cu = 0
        steps_run = 0
        events = []
        max_active = 0
        while pending or waiting or active:
            now = stamp()
            while pending and pending[0].arrival <= now:
                waiting.append(pending.popleft())
            if not active:
                self._admit(waiting, active, stamp)
                max_active = max(max_active, len(active))
                if not active:
                    # idle until the next arrival
                    if pending:
                        wait = pending[0].arrival - stamp()
                        if wait > 0:
                            time.sleep(min(wait / time_scale, 0.01))
                    continue
            # launch the batch up to the next completion (at most `chunk` steps) ...
            left = {mid: req.steps_left for mid, req in active.items()}
            n = max(1, min(self.chunk, min(left.values())))
            ev = (torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True))
            ev[0].record(self.stream)
            ens.step(n)
            ev[1].record(self.stream)
            events.append(ev)
            steps_run += n
            for req in active.values():   # the members of this chunk (admissions below join later)
                req.steps_left -= n
            # ... and while it runs, admit the arrivals (they join at the next step boundary)
            now = stamp()
            while pending and pending[0].arrival <= now:
                waiting.append(pending.popleft())
            self._admit(waiting, active, stamp)
            max_active = max(max_active, len(active))
            ens.sync()
            for mid in [mid for mid, req in active.items() if req.steps_left == 0]:
                req = active.pop(mid)
                if self.keep:
                    req.result = ens.download(mid)
                st = ens.status(mid)
                if st != 0:
                    raise RuntimeError(f"member {mid} (request {req.rid}) reported status {st}")
                ens.remove(mid)
                req.finished = stamp()
                total_cu += req.cell_updates
                done.append(req)
        wall = stamp()
        torch.cuda.synchronize()
        busy_s = sum(a.elapsed_time(b) for a, b in events) * 1e-3 * time_scale
        lat = np.array([r.finished - r.arrival for r in done])
        return dict(
            requests=len(done), wall_s=wall, busy_s=busy_s, batch_steps=steps_run, max_active=max_active,
            cell_updates=total_cu, cell_updates_per_s=total_cu / wall if wall > 0 else 0.0,
            p50_latency_s=float(np.percentile(lat, 50)) if len(lat) else math.nan,
            p99_latency_s=float(np.percentile(lat, 99)) if len(lat) else math.nan,
            mean_latency_s=float(lat.mean()) if len(lat) else math.nan,
            done=done)


def main(argv=None):
    """Serve seeded Poisson arrivals and print one JSON line: p50/p99 run latency and
    tracer cell-updates per second of wall time."""
    import argparse
    import json
    ap = argparse.ArgumentParser()
    ap.add_argument("--requests", type=int, default=2000)
    ap.add_argument("--rate", type=float, default=50.0, help="arrivals per second")
    ap.add_argument("--smin", type=int, default=200)
    ap.add_argument("--smax", type=int, default=5000)
    ap.add_argument("--chunk", type=int, default=25)
    ap.add_argument("--budget-gb", type=float, default=0.0, help="HBM budget (0: 90%% of free memory)")
    ap.add_argument("--seed", type=int, default=7)
    a = ap.parse_args(argv)
    reqs = poisson_requests(a.requests, rate=a.rate, seed=a.seed, smin=a.smin, smax=a.smax)
    srv = Server(hbm_budget_bytes=int(a.budget_gb * 1e9), chunk=a.chunk)
    st = srv.run(reqs)
    srv.close()
    st.pop("done")
    st.update(dict(arrival_rate=a.rate, steps_range=[a.smin, a.smax], chunk=a.chunk))
    print(json.dumps(st))


if __name__ == "__main__":
    main()
