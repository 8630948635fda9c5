"""Regenerate the golden fixtures of the rows next to the tracer step (this folder).

Each fixture holds the inputs and the oracle's outputs of one small case: the BIOGEM tracer
coupling (oracle/biogem_oracle.c, checked bit-identical against oracle/biogem_np.py), the EMBM
and sea-ice steppers (oracle/surface_oracle.c, checked against oracle/surface_np.py) and the
momentum step (oracle/momentum_oracle.c).  As for the tracer-step fixtures, no Fortran compiler
exists here: they pin the restatements against regressions, not against a run of the reference.
Run from the repository root:  python tests/golden/rows/make_golden_rows.py
"""
import json
import os
import sys

import numpy as np

ROOT = os.path.dirname(os.path.dirname(os.path.dirname(os.path.dirname(os.path.abspath(__file__)))))
sys.path.insert(0, ROOT)

from cgenie_gb300 import biogem, grid, momentum, surface  # noqa: E402
from oracle import biogem_np as bnp  # noqa: E402
from oracle import oracle_lib as ol  # noqa: E402
from oracle import surface_np as snp  # noqa: E402

HERE = os.path.dirname(os.path.abspath(__file__))


def coupling(name, kw, n_l_sed, force):
    m = grid.make_member(grid.MemberConfig(**kw))
    st = biogem.make_state(m, n_l_sed=n_l_sed, seed=3)
    go = ol.go_ts_interior(m.ts)
    a = st.copy()
    ts, _ = ol.bg_tracercoupling(m, a, go, force_ts=force)
    b = st.copy()
    g = np.ascontiguousarray(go.transpose(3, 2, 1, 0))
    o, _ = bnp.tracercoupling(g, b.vocn, b.mass, b.volume, b.rmass, b.vdocn, b.vbio_part, b.vdbio_part,
                              m.k1[1:-1, 1:-1].T, (biogem.CONST_ZEROC, biogem.SALN0), force)
    assert np.array_equal(o.transpose(3, 2, 1, 0), ts) and np.array_equal(a.vocn, b.vocn), name
    np.savez_compressed(os.path.join(HERE, name + ".npz"), kind="coupling", force=force, cfg=json.dumps(kw),
                        n_l_sed=n_l_sed,
                        maxi=m.maxi, maxj=m.maxj, maxk=m.maxk, k1=m.k1, go_ts=go,
                        **{"in_" + f: getattr(st, f) for f in ("vocn", "mass", "volume", "rmass", "vbio_part", "vdocn",
                                                               "vdbio_part")},
                        out_go_ts=ts, out_vocn=a.vocn, out_mass=a.mass, out_rmass=a.rmass, out_vbio_part=a.vbio_part)


def surf(name, kw, kind, nsteps):
    m = grid.make_member(grid.MemberConfig(**kw))
    c = surface.embm_case(m, seed=4) if kind == "embm" else surface.seaice_case(m, seed=4, explicit=kind == "ice_x")
    a = c.copy()
    ol.surface_step(a, nsteps)
    b = c.copy()
    if kind == "ice_x":
        snp.tstepsic(b.maxk, b.dt, b.rdphi, b.diffsic, b.tsc, b.sica_thresh, b.sich_thresh, b.rc, b.cv, b.rdsv, b.rds,
                     b.k1, b.tq, b.tq1, b.source, b.vel)
    else:
        snp.step(b.kind, b.maxk, b.dt, b.dphi, b.rdphi, b.betaz, b.betam, b.diffmod0, b.ppmin, b.ppmax, b.diffsic,
                 b.tsc, b.rc, b.cv, b.dsv, b.rdsv, b.rds, b.diffa, b.k1, b.tq, b.tq1, b.source, b.vel, b.pptn, nsteps)
    assert np.array_equal(a.tq, b.tq), name
    fields = {}
    for f in ("kind", "maxi", "maxj", "maxk", "dt", "dphi", "rdphi", "diffmod0", "ppmin", "ppmax", "diffsic", "tsc",
              "sica_thresh", "sich_thresh"):
        fields[f] = getattr(c, f)
    for f in ("rc", "cv", "dsv", "rdsv", "rds", "tq", "tq1", "source", "vel", "pptn", "diffa", "k1"):
        v = getattr(c, f)
        if v is not None:
            fields[f] = v
    np.savez_compressed(os.path.join(HERE, name + ".npz"), surface_kind=kind, nsteps=nsteps,
                        betaz=np.array(c.betaz), betam=np.array(c.betam), out_tq=a.tq, out_tq1=a.tq1, **fields)


def mom(name, kw, steps):
    m = grid.make_member(grid.MemberConfig(**kw))
    c = momentum.make_case(m, seed=5)
    o = ol.OracleMomentum(c)
    for _ in range(steps):
        o.step(m.rho)
    st = o.state()
    o.close()
    np.savez_compressed(os.path.join(HERE, name + ".npz"), kind="momentum", cfg=json.dumps(kw), steps=steps,
                        maxi=c.maxi, maxj=c.maxj,
                        maxk=c.maxk, isles=c.isles, mpi=c.mpi, dphi=c.dphi, rdphi=c.rdphi, rel=c.rel, rho=m.rho,
                        tau=c.tau, dztau=c.dztau, dztav=c.dztav, **{"a_" + k: v for k, v in c.arrays.items()},
                        out_u=st["u"], out_u1=st["u1"], out_ub=st["ub"], out_psi=st["psi"])


if __name__ == "__main__":
    coupling("coupling_12x10x8_l5", dict(maxi=12, maxj=10, maxk=8, maxl=5, seed=81), 3, False)
    coupling("coupling_force_ts_10x8x6_l4", dict(maxi=10, maxj=8, maxk=6, maxl=4, seed=82), 1, True)
    surf("embm_12x10", dict(maxi=12, maxj=10, maxk=4, maxl=2, seed=83), "embm", 3)
    surf("seaice_12x10", dict(maxi=12, maxj=10, maxk=6, maxl=2, seed=84), "ice", 1)
    surf("seaice_explicit_12x10", dict(maxi=12, maxj=10, maxk=6, maxl=2, seed=85), "ice_x", 1)
    mom("momentum_18x14x8_island", dict(maxi=18, maxj=14, maxk=8, maxl=2, seed=86, mask="basin_island"), 2)
    print("written")
