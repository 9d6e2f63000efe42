"""Multi-GPU host logic of bench.py (replicas, weak scaling) with world_size 2 over gloo on the CPU: the job time
is the slowest rank's, every rank solves its own ensemble, and the reference arm runs on rank 0 only."""
import os
import socket

import pytest
import torch.multiprocessing as mp


def _free_port():
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def _rank_main(rank, world, port, out):
    import sys
    import torch.distributed as dist
    sys.path.insert(0, os.path.dirname(os.path.dirname(os.path.abspath(__file__))))
    os.environ["MASTER_ADDR"] = "127.0.0.1"
    os.environ["MASTER_PORT"] = str(port)
    dist.init_process_group("gloo", rank=rank, world_size=world)
    try:
        import bench
        t = bench.max_over_ranks(1.5 + rank, dist, "cpu")          # rank r took 1.5 + r seconds
        seeds = bench.rank_seed0(rank)

        class A:
            warmup, steps = 1, 1
        rc = bench.run_reference(A, rank, world) if rank == 1 else 0  # rank 1 of the reference arm: no work
        out.put((rank, t, seeds, rc))
    finally:
        dist.destroy_process_group()


def test_two_ranks_over_gloo():
    ctx = mp.get_context("spawn")
    out = ctx.Queue()
    port = _free_port()
    procs = [ctx.Process(target=_rank_main, args=(r, 2, port, out)) for r in range(2)]
    for p in procs:
        p.start()
    for p in procs:
        p.join(timeout=180)
    assert all(p.exitcode == 0 for p in procs)
    res = sorted(out.get(timeout=5) for _ in range(2))
    assert [r[1] for r in res] == [2.5, 2.5]                        # max over ranks on every rank
    assert res[0][2] != res[1][2]                                   # distinct ensembles (weak scaling)
    assert res[1][3] == 0


def test_single_process_identity():
    import bench
    assert bench.max_over_ranks(3.25) == 3.25
    assert bench.rank_seed0(0) == 0 and bench.rank_seed0(3) == 192
