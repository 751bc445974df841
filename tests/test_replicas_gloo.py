"""The N>1 path of bench.py is replicas: every rank runs the same workload on
its own GPU, timing is max-over-ranks behind barriers, and no collective
touches the data path.  These tests drive that host logic with two gloo ranks
on the CPU (the per-rank perft here is the CPU oracle)."""
import os
import socket
import sys

import numpy as np
import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def _free_port():
    s = socket.socket()
    s.bind(("127.0.0.1", 0))
    p = s.getsockname()[1]
    s.close()
    return p


def _rank_main(rank, world, port, q):
    os.environ.update(RANK=str(rank), WORLD_SIZE=str(world), LOCAL_RANK=str(rank),
                      MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port))
    sys.path.insert(0, ROOT)
    import bench
    import oracle as O
    import torch.distributed as dist
    w, r, local, d = bench.dist_setup()
    assert (w, r) == (world, rank) and d is not None and dist.get_backend() == "gloo"
    bench.barrier(d)
    # each rank "times" a different duration; every rank must see the max
    elapsed = bench.max_over_ranks(d, 1.0 + rank)
    # replica workload: the same seeded positions on every rank
    orc = O.Oracle(1)
    boards, depths = orc.playouts(3, 16, 0, 60, 1, 2, 3, with_depths=True)
    out, _ = orc.perft_batch(boards, depths, 1)
    import torch
    mine = torch.tensor(out.astype(np.int64))
    gathered = [torch.zeros_like(mine) for _ in range(world)]
    dist.all_gather(gathered, mine)
    same = all(bool((g == gathered[0]).all()) for g in gathered)
    bench.barrier(d)
    dist.destroy_process_group()
    q.put((rank, elapsed, same, int(out.sum())))


@pytest.mark.timeout(120)
def test_two_gloo_ranks_barrier_max_and_identical_replicas():
    import multiprocessing as mp
    ctx = mp.get_context("spawn")
    q = ctx.Queue()
    port = _free_port()
    procs = [ctx.Process(target=_rank_main, args=(r, 2, port, q)) for r in range(2)]
    for p in procs:
        p.start()
    res = sorted(q.get(timeout=100) for _ in procs)
    for p in procs:
        p.join(timeout=30)
        assert p.exitcode == 0
    assert [r for r, *_ in res] == [0, 1]
    assert all(e == 2.0 for _, e, _, _ in res)
    assert all(same for _, _, same, _ in res)
    assert res[0][3] == res[1][3] > 0
