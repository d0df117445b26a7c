"""The multi-GPU path of bench.py, on CPU with two gloo ranks.

Chains are independent, so N GPUs run N replicas (one process per GPU,
each with its own Philox key) and no data path exchanges anything; the job's
figures are the slowest rank's time and the sum of every rank's moves.  This
file checks that reduction and the per-rank keys with world_size 2 over
gloo on 127.0.0.1, the way torchrun would start the ranks.
"""
import os
import socket
import sys

import pytest

REPO = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def _free_port():
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def _rank_main(rank, world, port, out):
    sys.path.insert(0, REPO)
    import torch
    import torch.distributed as dist
    os.environ.update(MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port))
    dist.init_process_group("gloo", rank=rank, world_size=world)
    import bench
    # rank r: time 10 + r ms, moves 1000 (r + 1), pairs 7 (r + 1)
    t, (moves, pairs) = bench.reduce_over_ranks(world, torch.device("cpu"), 10.0 + rank,
                                                [1000 * (rank + 1), 7 * (rank + 1)])

    class A:
        seed = 5
    out[rank] = (t, moves, pairs, bench.rank_seed(A, rank))
    dist.barrier()
    dist.destroy_process_group()


def test_reduce_over_ranks_two_gloo_ranks():
    torch = pytest.importorskip("torch")
    mp = torch.multiprocessing.get_context("spawn")
    with mp.Manager() as m:
        out = m.dict()
        port = _free_port()
        procs = [mp.Process(target=_rank_main, args=(r, 2, port, out)) for r in range(2)]
        for p in procs:
            p.start()
        for p in procs:
            p.join(timeout=120)
            assert p.exitcode == 0
        res = dict(out)
    for r in range(2):
        t, moves, pairs, seed = res[r]
        assert t == 11.0  # the slowest rank's time
        assert moves == 3000.0 and pairs == 21.0  # every rank's work counted once
    assert res[0][3] != res[1][3]  # each rank's chains have their own key


def test_single_rank_is_identity():
    sys.path.insert(0, REPO)
    import bench
    t, (a, b) = bench.reduce_over_ranks(1, None, 3.5, [10, 20])
    assert (t, a, b) == (3.5, 10.0, 20.0)
