"""Autotuner for the batched ensemble kernel: column-tile shape per grid shape.

A work item of the batched kernel is one TX x TY tile of water columns of one
member (TX*TY <= 128 threads).  The tile shape sets the halo overhead of the
shared-memory slabs ((TX+2)(TY+2)/(TX*TY)), the idle threads of partial
tiles, the shared memory per CTA (hence CTAs per SM) and the number of work
items available for load balance.  `tune()` times candidate shapes on a
synthetic ensemble of each grid shape with CUDA events and keeps the fastest;
the table is stored as JSON and applied by `Ensemble.add` through
gb_ens_set_tuning before each admission.
"""
from __future__ import annotations

import json
import os
import time
from typing import Dict, Iterable, Optional, Tuple

HERE = os.path.dirname(os.path.abspath(__file__))
TABLE_PATH = os.path.join(HERE, "tuning.json")

Shape = Tuple[int, int, int]

# a tuned tile replaces the planner's only when it is faster by more than run-to-run noise
NOISE = 1.02


def candidates(maxi: int, maxj: int):
    """Tile shapes worth timing: the patch planner's own choice, written (0, 0), then
    whole-row and near-square tiles of 64..128 columns."""
    out = set()
    for tx in range(4, min(64, maxi) + 1):
        for ty in range(1, min(32, maxj) + 1):
            n = tx * ty
            if n < 64 or n > 128:
                continue
            nti = -(-maxi // tx)
            ntj = -(-maxj // ty)
            util = maxi * maxj / (nti * ntj * n)
            halo = (tx + 2) * (ty + 2) / n
            if util >= 0.8 and halo <= 1.9:
                out.add((tx, ty))
    # keep the 8 best by a simple cost model (loads + idle threads)
    def cost(t):
        tx, ty = t
        nti, ntj = -(-maxi // tx), -(-maxj // ty)
        return nti * ntj * (tx + 2) * (ty + 2) + 0.5 * (nti * ntj * tx * ty - maxi * maxj)
    return [(0, 0)] + sorted(out, key=cost)[:8]


def load_table(path: str = TABLE_PATH) -> Dict[str, list]:
    try:
        with open(path) as f:
            return json.load(f)
    except (OSError, ValueError):
        return {}


def lookup(table: Dict[str, list], maxi: int, maxj: int, maxk: int) -> Optional[Tuple[int, int]]:
    """The stored tile of a grid shape; None when none is stored or the planner's own choice
    (stored as 0, 0) won."""
    v = table.get(f"{maxi}x{maxj}x{maxk}")
    return (int(v[0]), int(v[1])) if v and (int(v[0]), int(v[1])) != (0, 0) else None


BATCH_KEY = "batch"   # [packing, ctas_per_sm, rate]: the launch-wide settings of a mixed batch


def batch_entry(table: Dict[str, list]) -> Tuple[int, int]:
    """The autotuned member packing and CTA cap of the batch, (0, 0) when none is stored."""
    v = table.get(BATCH_KEY)
    return (int(v[0]), int(v[1])) if v else (0, 0)


def make_members(shape: Shape, members: int = 64, seed: int = 5):
    """Seeded members of one grid shape with 2-24 tracers (the ensemble's mix)."""
    import numpy as np
    from . import grid
    rng = np.random.default_rng(seed)
    return [grid.make_member(grid.MemberConfig(maxi=shape[0], maxj=shape[1], maxk=shape[2],
                                               maxl=int(rng.integers(2, 25)), seed=int(rng.integers(0, 2**31 - 1)),
                                               tracer_kind="bgc"))
            for _ in range(members)]


def time_shape(mems, tile: Tuple[int, int], steps: int = 30, packing: int = 0, ctas_per_sm: int = 0,
               use_table: bool = False) -> float:
    """Tracer cell-updates/s of the batched step (CUDA graph) on `mems` with one tile shape
    ((0, 0) with use_table: the table's tiles per member), member packing and CTA cap; 0 when
    the shape does not fit the kernel limits on some member."""
    from .ensemble import Ensemble
    ens = Ensemble(tile_i=tile[0], tile_j=tile[1], use_graph=True, use_table=use_table, packing=packing,
                   ctas_per_sm=ctas_per_sm)
    try:
        ens.add_many(mems)
    except Exception:
        ens.close()
        return 0.0
    ens.step(steps)     # capture the graph, warm up
    ens.sync()
    t0 = time.perf_counter()
    ens.step(steps)
    ens.sync()
    dt = time.perf_counter() - t0
    cu = sum(m.wet_cells * m.maxl for m in mems) * steps
    ens.close()
    return cu / dt


def tune(shapes: Iterable[Shape] = ((18, 18, 16), (36, 36, 16), (36, 36, 32)), members: int = 64,
         steps: int = 30, path: str = TABLE_PATH, verbose: bool = True) -> Dict[str, list]:
    """Time every candidate tile of each shape (the planner's choice included) and store, per
    shape, the best tile when it beats the planner's by more than run-to-run noise, else the
    planner's (0, 0); with the rate."""
    table = load_table(path)
    for shape in shapes:
        mems = make_members(shape, members)
        best = None
        rates = []
        for tile in candidates(shape[0], shape[1]):
            rate = time_shape(mems, tile, steps=steps)
            rates.append((tile, rate))
            if verbose:
                print(f"{shape} tile {tile}: {rate:.3e} cell-updates/s", flush=True)
            if best is None or rate > best[1]:
                best = (tile, rate)
        key = f"{shape[0]}x{shape[1]}x{shape[2]}"
        planner = next(r for t, r in rates if t == (0, 0))
        if best[0] == (0, 0) or best[1] < NOISE * planner:
            table[key] = [0, 0, planner]     # the planner's choice is as good
        else:
            table[key] = [best[0][0], best[0][1], best[1]]
        if verbose:
            print(f"{shape}: best tile {best[0]} ({best[1]:.3e})", flush=True)
    with open(path, "w") as f:
        json.dump(table, f, indent=1, sort_keys=True)
    return table


def tune_batch(members: int = 96, steps: int = 30, path: str = TABLE_PATH, verbose: bool = True,
               packings: Iterable[int] = (0, 1, 2), caps: Iterable[int] = (0, 3, 4)) -> Dict[str, list]:
    """Member packing and CTA cap of a mixed batch (the three grid shapes, 2-24 tracers, the
    stored tiles): every combination is timed; the best is stored when it beats the default
    (members packed together, no cap) by more than run-to-run noise, else the default."""
    table = load_table(path)
    shapes = ((18, 18, 16), (36, 36, 16), (36, 36, 32))
    mems = []
    for n, shape in enumerate(shapes):
        mems += make_members(shape, members // len(shapes), seed=11 + n)
    rates = {}
    for pk in packings:
        for cap in caps:
            rates[(pk, cap)] = time_shape(mems, (0, 0), steps=steps, packing=pk, ctas_per_sm=cap, use_table=True)
            if verbose:
                print(f"packing {pk} ctas_per_sm {cap}: {rates[(pk, cap)]:.3e} cell-updates/s", flush=True)
    best = max(rates, key=rates.get)
    if best == (0, 0) or rates[best] < NOISE * rates[(0, 0)]:
        best = (0, 0)
    table[BATCH_KEY] = [best[0], best[1], rates[best]]
    with open(path, "w") as f:
        json.dump(table, f, indent=1, sort_keys=True)
    if verbose:
        print(f"batch: best packing {best[0]}, ctas_per_sm {best[1]} ({rates[best]:.3e})", flush=True)
    return table


if __name__ == "__main__":
    import sys
    if "--batch" in sys.argv:
        tune_batch()
    else:
        tune()
