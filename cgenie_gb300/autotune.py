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


def candidates(maxi: int, maxj: int):
    """Tile shapes worth timing: whole-row tiles, near-square tiles and the
    default cost-model choice, all with 64..128 threads."""
    out = set()
    for tx in range(4, 65):
        for ty in range(1, 33):
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
    return sorted(out, key=cost)[:8]


def load_table(path: str = TABLE_PATH) -> Dict[str, list]:
    try:
        with open(path) as f:
            return json.load(f)
    except (OSError, ValueError):
        return {}


def lookup(table: Dict[str, list], maxi: int, maxj: int, maxk: int) -> Optional[Tuple[int, int]]:
    v = table.get(f"{maxi}x{maxj}x{maxk}")
    return (int(v[0]), int(v[1])) if v else None


def time_shape(shape: Shape, tile: Tuple[int, int], members: int = 48, steps: int = 10, seed: int = 5,
               lmean: int = 13) -> float:
    """Tracer cell-updates/s of the batched kernel for `members` copies of one shape."""
    import numpy as np
    import torch
    from . import grid
    from .ensemble import Ensemble
    rng = np.random.default_rng(seed)
    mems = []
    for n in range(members):
        cfg = grid.MemberConfig(maxi=shape[0], maxj=shape[1], maxk=shape[2], maxl=int(rng.integers(2, 25)),
                                seed=int(rng.integers(0, 2**31 - 1)), tracer_kind="bgc")
        mems.append(grid.make_member(cfg))
    ens = Ensemble(tile_i=tile[0], tile_j=tile[1])
    for m in mems:
        ens.add(m)
    ens.step(3)
    ens.sync()
    s = torch.cuda.Event(enable_timing=True)
    e = torch.cuda.Event(enable_timing=True)
    t0 = time.perf_counter()
    ens.step(steps)
    ens.sync()
    dt = time.perf_counter() - t0
    cu = sum(m.wet_cells * m.maxl for m in mems) * steps
    ens.close()
    del s, e
    return cu / dt


def tune(shapes: Iterable[Shape] = ((18, 18, 16), (36, 36, 16), (36, 36, 32)), members: int = 48,
         steps: int = 10, path: str = TABLE_PATH, verbose: bool = True) -> Dict[str, list]:
    table = load_table(path)
    for shape in shapes:
        best = None
        for tile in candidates(shape[0], shape[1]):
            rate = time_shape(shape, tile, members=members, steps=steps)
            if verbose:
                print(f"{shape} tile {tile}: {rate:.3e} cell-updates/s", flush=True)
            if best is None or rate > best[1]:
                best = (tile, rate)
        table[f"{shape[0]}x{shape[1]}x{shape[2]}"] = [best[0][0], best[0][1], best[1]]
        if verbose:
            print(f"{shape}: best tile {best[0]} ({best[1]:.3e})", flush=True)
    with open(path, "w") as f:
        json.dump(table, f, indent=1, sort_keys=True)
    return table


if __name__ == "__main__":
    tune()
