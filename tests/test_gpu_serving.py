"""Serving loop on the GPU: requests that arrive while others run are admitted into the
running batch (continuous batching), every result equals the same member run alone (bit
for bit), and admission respects the HBM budget."""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def test_continuous_batching_results_equal_alone(gpu_lib):
    from cgenie_gb300.ensemble import Ensemble
    from cgenie_gb300.serving import MemberFactory, Server, poisson_requests
    fac = MemberFactory(variants=2)
    reqs = poisson_requests(10, rate=400.0, seed=5, smin=20, smax=80)
    srv = Server(chunk=6, keep_results=True, factory=fac)
    st = srv.run(reqs)
    srv.close()
    done = st["done"]
    assert st["requests"] == len(reqs)
    # admissions happened while other runs were in flight
    overlapped = sum(1 for a in done for b in done
                     if a is not b and b.admitted < a.admitted < b.finished)
    assert overlapped > 0
    assert st["max_active"] > 1
    for r in done:
        ens = Ensemble()
        mid = ens.add(fac.member(r), steps=r.steps)
        ens.step(r.steps)
        alone = ens.download(mid)
        ens.close()
        assert np.array_equal(alone["ts"], r.result["ts"]), r.rid
        assert np.array_equal(alone["cost"], r.result["cost"]), r.rid


def test_admission_waits_for_budget(gpu_lib):
    from cgenie_gb300.ensemble import Ensemble
    from cgenie_gb300.serving import MemberFactory, Server, poisson_requests
    fac = MemberFactory(variants=1)
    reqs = poisson_requests(6, rate=1000.0, seed=9, smin=10, smax=30)
    for r in reqs:                      # one size: the budget holds two members
        r.shape, r.maxl = (36, 36, 16), 8
    size = Ensemble.member_bytes(fac.member(reqs[0]))
    srv = Server(hbm_budget_bytes=int(2.5 * size), chunk=5, factory=fac)
    st = srv.run(reqs)
    srv.close()
    assert st["requests"] == len(reqs)
    assert 1 <= st["max_active"] <= 2
    assert st["p99_latency_s"] >= st["p50_latency_s"] > 0
