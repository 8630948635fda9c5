"""Save / load a synthetic member (inputs) and oracle outputs as .npz fixtures."""
import dataclasses
import json

import numpy as np

from cgenie_gb300 import grid

ARRAYS = ["diff", "ec", "rc", "rc2", "cv", "cv2", "dsv", "rdsv", "ds", "rds", "dz", "dza", "rdz", "rdza",
          "zro", "dt", "zw", "ssmax", "ediff1", "diffmax", "k1", "ts", "ts1", "rho", "u", "cost", "icosd"]
SCALARS = ["maxi", "maxj", "maxk", "maxl", "ediff0", "ediffpow2", "ediffpow2i", "dphi", "rdphi"]
OPTIONAL = ["mlddec", "mlddecd", "mldketau", "mld", "mldk"]   # mixed-layer scheme inputs/state


def save(path, m, outputs=None):
    d = {f"in_{a}": getattr(m, a) for a in ARRAYS}
    d.update({f"in_{a}": getattr(m, a) for a in OPTIONAL if getattr(m, a, None) is not None})
    meta = {s: (getattr(m, s).item() if hasattr(getattr(m, s), "item") else getattr(m, s)) for s in SCALARS}
    meta["cfg"] = dataclasses.asdict(m.cfg)
    d["meta"] = np.array(json.dumps(meta))
    for k, v in (outputs or {}).items():
        d[f"out_{k}"] = np.asarray(v)
    np.savez_compressed(path, **d)


def load(path):
    z = np.load(path)
    meta = json.loads(str(z["meta"]))
    cfg = grid.MemberConfig(**meta.pop("cfg"))
    kw = {a: z[f"in_{a}"].copy() for a in ARRAYS}
    kw.update({a: z[f"in_{a}"].copy() for a in OPTIONAL if f"in_{a}" in z.files})
    m = grid.Member(cfg=cfg, **meta, **kw)
    outs = {k[4:]: z[k] for k in z.files if k.startswith("out_")}
    return m, outs
