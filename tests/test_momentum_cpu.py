"""CPU checks of the momentum-step restatement (oracle/momentum_oracle.c: invert, ubarsolv,
island, matinv_gold, matmult, wind, jbar, velc of src/goldstein/goldstein.f90 and
goldstein_lib.f90): the banded LU solve against a dense solve of the assembled matrix, and
the boundary and island conditions the reference's streamfunction satisfies."""
import numpy as np
import pytest

from cgenie_gb300 import grid, momentum
from oracle import oracle_lib as ol


@pytest.mark.parametrize("mask", ["basin", "basin_island"])
def test_unit_source_solves_match_dense_solve(mask):
    m = grid.make_member(grid.MemberConfig(maxi=18, maxj=14, maxk=8, maxl=2, seed=1, mask=mask))
    c = momentum.make_case(m, seed=2)
    o = ol.OracleMomentum(c)
    A = o.matrix()
    psisl, _, _ = o.islands()
    lab = c.arrays["psiles"].reshape(c.maxj + 1, c.maxi)
    for isol in range(c.isles):
        b = (lab == isol + 2).astype(float).reshape(-1)
        x = np.linalg.solve(A, b).reshape(c.maxj + 1, c.maxi)
        np.testing.assert_allclose(psisl[isol][:, 1:], x, rtol=0, atol=1e-12 * np.abs(x).max())
        np.testing.assert_array_equal(psisl[isol][:, 0], psisl[isol][:, -1])   # psi(0,j) = psi(maxi,j)


@pytest.mark.parametrize("mask", ["basin", "basin_island"])
def test_step_streamfunction_conditions(mask):
    """After a step psi is 0 on the first landmass and constant (psibc) on each island: the
    trivial equations at dry psi points carry no forcing, and the island corrections add
    psibc times a unit solution that is 1 on its island and 0 on the others."""
    m = grid.make_member(grid.MemberConfig(maxi=18, maxj=14, maxk=8, maxl=2, seed=3, mask=mask))
    c = momentum.make_case(m, seed=4)
    o = ol.OracleMomentum(c)
    o.step(m.rho)
    st = o.state()
    lab = c.arrays["psiles"].reshape(c.maxj + 1, c.maxi)
    psi = st["psi"][:, 1:]
    assert np.all(psi[lab == 1] == 0.0)
    for isl in range(c.isles):
        v = psi[lab == isl + 2]
        assert v.min() == v.max() and v[0] != 0.0
    # w from continuity: the column integral of the horizontal divergence
    assert np.isfinite(st["u"]).all() and np.abs(st["u"]).max() > 0


def test_oracle_header_cites_reference():
    import os
    src = open(os.path.join(os.path.dirname(os.path.dirname(os.path.abspath(__file__))), "oracle",
                            "momentum_oracle.c")).read()
    assert "ORACLE -- test infrastructure only" in src
    assert "goldstein.f90:3500-3565" in src and "goldstein_lib.f90:186-241" in src
    assert "parity unpinned" in src
