"""The oracles of the rows next to the tracer step reproduce their committed fixtures
(tests/golden/rows): the BIOGEM coupling and the surface steppers bit for bit, the momentum
step bit for bit (the oracle is the reference's banded LU path).  The seeded generators must
still produce the fixtures' inputs."""
import os

import numpy as np
import pytest

import rows_io
from oracle import oracle_lib as ol


@pytest.mark.parametrize("path", rows_io.paths("coupling"), ids=lambda p: os.path.basename(p)[:-4])
def test_coupling_fixture(path):
    z, m, st = rows_io.load_coupling(path)
    assert np.array_equal(m.k1, z["k1"]) and np.array_equal(ol.go_ts_interior(m.ts), z["go_ts"])
    ts, _ = ol.bg_tracercoupling(m, st, np.array(z["go_ts"]), force_ts=bool(z["force"]))
    assert np.array_equal(ts, z["out_go_ts"])
    for f in ("vocn", "mass", "rmass", "vbio_part"):
        assert np.array_equal(getattr(st, f), z["out_" + f]), f


@pytest.mark.parametrize("path", rows_io.paths("embm") + rows_io.paths("seaice"), ids=lambda p: os.path.basename(p)[:-4])
def test_surface_fixture(path):
    z, c = rows_io.load_surface(path)
    ol.surface_step(c, int(z["nsteps"]))
    assert np.array_equal(c.tq, z["out_tq"]) and np.array_equal(c.tq1, z["out_tq1"])


@pytest.mark.parametrize("path", rows_io.paths("momentum"), ids=lambda p: os.path.basename(p)[:-4])
def test_momentum_fixture(path):
    z, m, c = rows_io.load_momentum(path)
    assert np.array_equal(m.rho, z["rho"])
    o = ol.OracleMomentum(c)
    for _ in range(int(z["steps"])):
        o.step(m.rho)
    st = o.state()
    for f in ("u", "u1", "ub", "psi"):
        assert np.array_equal(st[f], z["out_" + f]), f
    o.close()
