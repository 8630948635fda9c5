"""Failure detection in the batched ensemble, by host-side injection (no device fault):
a member admitted with a non-finite value in a wet cell reports status bit 0 (non-finite
state) after its steps, while the members stepped in the same batch report 0 and end
bit-identical to their runs alone; the member can then be retired without stopping the
batch.  The reference stops the whole run instead (die -> STOP,
src/wrappers/genie_util.f90:14-30; the diag2 crash barrier, goldstein_diag.f90:48-54)."""
import dataclasses

import numpy as np
import pytest

from cgenie_gb300 import grid

pytestmark = pytest.mark.gpu


def test_nonfinite_member_is_flagged_and_isolated(gpu_lib):
    from cgenie_gb300.ensemble import Ensemble
    cfgs = grid.ensemble_configs(3, seed=13, lmin=3, lmax=10)
    mems = [grid.make_member(c) for c in cfgs]
    m = mems[1]
    ts = m.ts.copy()
    j, i = np.argwhere(m.k1[1:-1, 1:-1] <= m.maxk)[0] + 1
    ts[m.maxk, j, i, 2] = np.nan                 # one wet surface cell of a tracer group
    bad = dataclasses.replace(m, ts=ts, ts1=ts.copy())
    ens = Ensemble(use_graph=True)
    ids = [ens.add(x) for x in (mems[0], bad, mems[2])]
    ens.step(8)
    st = [ens.status(i_) for i_ in ids]
    assert st[1] & 1, st
    assert st[0] == 0 and st[2] == 0, st
    outs = {n: ens.download(ids[n])["ts"] for n in (0, 2)}
    ens.remove(ids[1])                           # retired; the batch goes on
    ens.step(2)
    assert ens.count()[0] == 2
    ens.close()
    for n in (0, 2):
        solo = Ensemble(use_graph=True)
        sid = solo.add(mems[n])
        solo.step(8)
        assert np.array_equal(solo.download(sid)["ts"], outs[n]), n
        solo.close()
