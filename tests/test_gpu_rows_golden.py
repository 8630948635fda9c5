"""The device paths of the rows next to the tracer step against their committed fixtures
(tests/golden/rows): the BIOGEM coupling and the surface steppers bit for bit, the momentum
step within 1e-9 (its streamfunction is inverse x right-hand side)."""
import os

import numpy as np
import pytest

import rows_io
from cgenie_gb300 import biogem, momentum, surface

pytestmark = pytest.mark.gpu


@pytest.mark.parametrize("path", rows_io.paths("coupling"), ids=lambda p: os.path.basename(p)[:-4])
def test_coupling_fixture(gpu_lib, path):
    from cgenie_gb300.goldstein import new_member_run
    z, m, st = rows_io.load_coupling(path)
    g = new_member_run(m)
    bg = biogem.BiogemCoupling(m, n_l_sed=int(z["n_l_sed"]), force_ts=bool(z["force"]))
    bg.upload(st)
    bg.set_increments(st)
    bg.tracercoupling(g)
    out = g.download()
    vocn, mass, rmass, vbio = bg.download()
    assert np.array_equal(out["ts"][1:m.maxk + 1, 1:-1, 1:-1, :], z["out_go_ts"])
    assert np.array_equal(vocn, z["out_vocn"]) and np.array_equal(mass, z["out_mass"])
    assert np.array_equal(rmass, z["out_rmass"]) and np.array_equal(vbio, z["out_vbio_part"])
    bg.close()
    g.close()


@pytest.mark.parametrize("path", rows_io.paths("embm") + rows_io.paths("seaice"), ids=lambda p: os.path.basename(p)[:-4])
def test_surface_fixture(gpu_lib, path):
    z, c = rows_io.load_surface(path)
    s = surface.SurfaceStepper(c)
    s.upload_state()
    s.set_forcing()
    s.step(int(z["nsteps"]))
    tq, tq1 = s.download()
    s.close()
    assert np.array_equal(tq, z["out_tq"]) and np.array_equal(tq1, z["out_tq1"])


@pytest.mark.parametrize("path", rows_io.paths("momentum"), ids=lambda p: os.path.basename(p)[:-4])
def test_momentum_fixture(gpu_lib, path):
    from cgenie_gb300.goldstein import new_member_run
    z, m, c = rows_io.load_momentum(path)
    g = new_member_run(m)
    mo = momentum.Momentum(c)
    mo.set_wind()
    for _ in range(int(z["steps"])):
        mo.step(g)
    out = mo.download()
    for f in ("u", "u1", "ub", "psi"):
        ref = z["out_" + f]
        assert np.abs(out[f] - ref).max() <= 1e-9 * np.abs(ref).max(), f
    mo.close()
    g.close()
