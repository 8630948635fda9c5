"""Loaders of the fixtures in tests/golden/rows (made by tests/golden/rows/make_golden_rows.py)."""
import glob
import json
import os

import numpy as np

from cgenie_gb300 import biogem, grid, momentum, surface

HERE = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden", "rows")


def paths(prefix):
    return sorted(glob.glob(os.path.join(HERE, prefix + "*.npz")))


def load_coupling(path):
    z = np.load(path)
    m = grid.make_member(grid.MemberConfig(**json.loads(str(z["cfg"]))))
    st = biogem.BiogemState(*(np.array(z["in_" + f]) for f in ("vocn", "mass", "volume", "rmass", "vbio_part",
                                                              "vdocn", "vdbio_part")))
    return z, m, st


def load_surface(path):
    z = np.load(path)
    kw = {f: (z[f].item() if z[f].shape == () else np.array(z[f])) for f in z.files
          if f not in ("surface_kind", "nsteps", "out_tq", "out_tq1", "betaz", "betam")}
    c = surface.SurfaceCase(betaz=tuple(z["betaz"]), betam=tuple(z["betam"]), **kw)
    return z, c


def load_momentum(path):
    z = np.load(path)
    m = grid.make_member(grid.MemberConfig(**json.loads(str(z["cfg"]))))
    arrays = {f[2:]: np.array(z[f]) for f in z.files if f.startswith("a_")}
    c = momentum.MomentumCase(maxi=int(z["maxi"]), maxj=int(z["maxj"]), maxk=int(z["maxk"]), isles=int(z["isles"]),
                              mpi=int(z["mpi"]), dphi=float(z["dphi"]), rdphi=float(z["rdphi"]), rel=float(z["rel"]),
                              arrays=arrays, tau=np.array(z["tau"]), dztau=np.array(z["dztau"]),
                              dztav=np.array(z["dztav"]))
    return z, m, c
