"""Regenerate the golden fixtures in this folder.

The reference tracer step cannot be compiled here (no Fortran compiler), so
these fixtures pin the oracle's results: every case was produced by the C
restatement (oracle/goldstein_oracle.c) and checked bit-identical against the
independent NumPy restatement (oracle/goldstein_np.py) before being written.
Run from the repository root:  python tests/golden/make_golden.py
(The fixtures of the BIOGEM coupling, the surface steppers and the momentum step are in
rows/, made by rows/make_golden_rows.py.)
"""
import os
import sys

import numpy as np

ROOT = os.path.dirname(os.path.dirname(os.path.dirname(os.path.abspath(__file__))))
sys.path.insert(0, ROOT)
sys.path.insert(0, os.path.join(ROOT, "tests"))

from cgenie_gb300 import grid  # noqa: E402
from oracle import goldstein_np as gnp  # noqa: E402
from oracle import oracle_lib  # noqa: E402
import member_io  # noqa: E402

HERE = os.path.dirname(os.path.abspath(__file__))

CASES = {
    # name: (config kwargs, steps)
    "plain_12x10x8_l3": (dict(maxi=12, maxj=10, maxk=8, maxl=3, seed=11), 6),
    "diso_12x10x8_l4": (dict(maxi=12, maxj=10, maxk=8, maxl=4, seed=12, diso=True, slope_max=1e-3), 6),
    "diso_ieos_12x10x8_l2": (dict(maxi=12, maxj=10, maxk=8, maxl=2, seed=13, diso=True, ieos=1), 5),
    "coshuffle_10x8x6_l3": (dict(maxi=10, maxj=8, maxk=6, maxl=3, seed=14, iconv=1, noise=2.0), 5),
    "coshuffle_ieos_10x8x6_l2": (dict(maxi=10, maxj=8, maxk=6, maxl=2, seed=15, iconv=1, ieos=1, noise=2.0), 5),
    "ediff_10x8x6_l3": (dict(maxi=10, maxj=8, maxk=6, maxl=3, seed=16, iediff=1, ediffpow2=1.0, diso=True), 5),
    "forcing_land94_9x7x5_l2": (dict(maxi=9, maxj=7, maxk=5, maxl=2, seed=17, forcing=1.0, land_code=94), 5),
    "mld_12x10x10_l3": (dict(maxi=12, maxj=10, maxk=10, maxl=3, seed=18, forcing=1.0, imld=1,
                             mldketau_max=3e-3, mldwindkedec=500.0), 5),
    "mld_ieos_coshuffle_12x10x10_l3": (dict(maxi=12, maxj=10, maxk=10, maxl=3, seed=19, forcing=1.0, imld=1,
                                            ieos=1, iconv=1, noise=2.0, mldketau_max=1e-2,
                                            mldwindkedec=2000.0), 5),
}


def make(name, kw, steps):
    cfg = grid.MemberConfig(**kw)
    m = grid.make_member(cfg)
    s = oracle_lib.OracleState(m)
    s.step(steps)
    p = gnp.Params(m, cfg.diso, cfg.ieos, cfg.iconv, cfg.iediff, cfg.imld)
    ts, ts1, rho, cost, icosd = m.copy_state()
    mld, mldk = m.mld.copy(), m.mldk.copy()
    dmax, limps = gnp.tstepo(m, p, ts, ts1, rho, m.u, cost, icosd, steps, mld, mldk)
    for a, b in [(s.ts, ts), (s.ts1, ts1), (s.rho, rho), (s.cost, cost), (s.icosd, icosd), (s.mld, mld),
                 (s.mldk, mldk)]:
        assert np.array_equal(a, b), name
    assert dmax == s.dmax.value and limps == s.limps.value, name
    outs = dict(steps=steps, ts=s.ts, ts1=s.ts1, rho=s.rho, cost=s.cost, icosd=s.icosd, dmax=s.dmax.value,
                limps=s.limps.value, inventory=s.inventory())
    if cfg.imld:
        outs.update(mld=s.mld, mldk=s.mldk)
    member_io.save(os.path.join(HERE, name + ".npz"), m, outs)


if __name__ == "__main__":
    only = sys.argv[1:]
    for name, (kw, steps) in CASES.items():
        if only and name not in only:
            continue
        make(name, kw, steps)
        print("wrote", name)
