"""Multi-rank host logic on CPU (gloo, world size 2): one ensemble is partitioned across the
ranks (rank r takes members r::2), each rank advances its members (with the oracle standing
in for the device step), the results are gathered on rank 0 in member order, and the job time
and work are reduced over ranks as the benchmark does under torchrun."""
import os
import socket
import sys

import numpy as np
import pytest

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(HERE)
N_MEMBERS = 5


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
    import torch.distributed as dist
    from cgenie_gb300 import grid
    from cgenie_gb300.replicas import gather, job_time, job_units, partition
    from oracle import oracle_lib
    dist.init_process_group("gloo", rank=rank, world_size=world)
    cfgs = grid.ensemble_configs(N_MEMBERS, seed=3, lmax=6)
    mine = partition(N_MEMBERS, rank, world)
    t0 = time.perf_counter()
    units = 0
    local = {}
    for i in mine:
        m = grid.make_member(cfgs[i])
        s = oracle_lib.OracleState(m)
        s.step(2)
        units += 2 * m.wet_cells * m.maxl
        local[i] = (s.ts.copy(), s.cost.copy())
    elapsed = time.perf_counter() - t0 + 0.05 * rank      # the second rank is slower
    tmax = job_time(elapsed, dist)
    total = job_units(units, dist)
    allres = gather(local, N_MEMBERS, dist)
    if rank == 0:
        np.savez(os.path.join(os.environ["GB_TEST_OUT"], "gathered.npz"),
                 **{f"ts{i}": r[0] for i, r in enumerate(allres)}, **{f"cost{i}": r[1] for i, r in enumerate(allres)})
    q.put((rank, elapsed, tmax, units, total, mine, allres is None))
    dist.barrier()
    dist.destroy_process_group()


def test_two_ranks_partition_gather_and_reduce(tmp_path):
    import multiprocessing as mp
    os.environ["GB_TEST_OUT"] = str(tmp_path)
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
    (r0, l0, t0, u0, s0, m0, n0), (r1, l1, t1, u1, s1, m1, n1) = out
    assert t0 == t1 == pytest.approx(max(l0, l1))
    assert s0 == s1 == u0 + u1
    assert m0 == [0, 2, 4] and m1 == [1, 3]          # the partition: members r::2
    assert not n0 and n1                             # gathered on rank 0 only
    # the gathered results are each member's own run, in member order
    sys.path.insert(0, ROOT)
    from cgenie_gb300 import grid
    from oracle import oracle_lib
    oracle_lib.build()
    got = np.load(os.path.join(str(tmp_path), "gathered.npz"))
    for i, c in enumerate(grid.ensemble_configs(N_MEMBERS, seed=3, lmax=6)):
        s = oracle_lib.OracleState(grid.make_member(c))
        s.step(2)
        assert np.array_equal(got[f"ts{i}"], s.ts) and np.array_equal(got[f"cost{i}"], s.cost)


def test_single_process_partition_and_reductions():
    sys.path.insert(0, ROOT)
    from cgenie_gb300.replicas import gather, job_time, job_units, partition
    assert job_time(1.5) == 1.5
    assert job_units(7) == 7
    assert partition(5, 0, 1) == [0, 1, 2, 3, 4]
    assert partition(7, 2, 3) == [2, 5]
    with pytest.raises(ValueError):
        partition(4, 2, 2)
    assert gather({1: "b", 0: "a"}, 2) == ["a", "b"]
    with pytest.raises(ValueError):
        gather({0: "a"}, 2)
