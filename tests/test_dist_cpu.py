"""Multi-rank host logic on CPU (gloo, world size 2): each rank builds its own members,
advances them with the oracle, and the job time and work are reduced over ranks as the
benchmark does under torchrun."""
import os
import socket
import sys

import pytest

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(HERE)


def _free_port():
    s = socket.socket()
    s.bind(("127.0.0.1", 0))
    p = s.getsockname()[1]
    s.close()
    return p


def _rank(rank, world, port, q):
    sys.path.insert(0, ROOT)
    os.environ.update(MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port))
    import time
    import numpy as np
    import torch.distributed as dist
    from cgenie_gb300 import grid
    from cgenie_gb300.replicas import job_time, job_units, rank_seed
    from oracle import oracle_lib
    dist.init_process_group("gloo", rank=rank, world_size=world)
    cfgs = grid.ensemble_configs(3, seed=rank_seed(3, rank))
    mems = [grid.make_member(c) for c in cfgs[:2]]
    t0 = time.perf_counter()
    units = 0
    for m in mems:
        s = oracle_lib.OracleState(m)
        s.step(2)
        units += 2 * m.wet_cells * m.maxl
    local = time.perf_counter() - t0 + 0.05 * rank      # the second rank is slower
    tmax = job_time(local, dist)
    total = job_units(units, dist)
    q.put((rank, local, tmax, units, total, float(np.sum(mems[0].k1))))
    dist.barrier()
    dist.destroy_process_group()


def test_two_ranks_reduce_time_and_work():
    import multiprocessing as mp
    ctx = mp.get_context("spawn")
    q = ctx.Queue()
    port = _free_port()
    ps = [ctx.Process(target=_rank, args=(r, 2, port, q)) for r in range(2)]
    for p in ps:
        p.start()
    out = sorted(q.get(timeout=240) for _ in ps)
    for p in ps:
        p.join(timeout=60)
        assert p.exitcode == 0
    (r0, l0, t0, u0, s0, k0), (r1, l1, t1, u1, s1, k1) = out
    assert t0 == t1 == pytest.approx(max(l0, l1))
    assert s0 == s1 == u0 + u1
    assert k0 != k1          # the ranks advance different members


def test_single_process_reductions_are_local():
    sys.path.insert(0, ROOT)
    from cgenie_gb300.replicas import job_time, job_units, rank_seed
    assert job_time(1.5) == 1.5
    assert job_units(7) == 7
    assert rank_seed(3, 0) == 3 and rank_seed(3, 1) != 3
