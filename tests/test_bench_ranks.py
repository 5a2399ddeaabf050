"""The multi-rank bench path on CPU: two gloo ranks shard the queries into
disjoint seed ranges and agree on the whole-job figures (the slowest rank's
time, the total solved)."""
import os
import socket

import pytest


def _free_port():
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def _rank(rank, world, port, out):
    import torch.distributed as dist
    os.environ.update(MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port))
    dist.init_process_group("gloo", rank=rank, world_size=world)
    import bench
    t, solved = bench.reduce_over_ranks(0.25 + 0.5 * rank, 100 + rank, world)
    out.put((rank, t, solved, bench.shard_seed0(rank, 1024, 5)))
    dist.destroy_process_group()


def test_two_gloo_ranks_reduce_and_shard():
    torch = pytest.importorskip("torch")
    import torch.multiprocessing as mp
    ctx = mp.get_context("spawn")
    q = ctx.Queue()
    port = _free_port()
    procs = [ctx.Process(target=_rank, args=(r, 2, port, q)) for r in range(2)]
    for p in procs:
        p.start()
    got = sorted(q.get(timeout=120) for _ in procs)
    for p in procs:
        p.join(timeout=60)
        assert p.exitcode == 0
    for rank, t, solved, seed0 in got:
        assert t == 0.75 and solved == 201       # max time, summed queries
    assert got[0][3] == 0 and got[1][3] == 5120  # disjoint query seeds: [0, 5120) and [5120, 10240)


def test_single_rank_is_identity():
    import bench
    assert bench.reduce_over_ranks(1.5, 7, 1) == (1.5, 7)
