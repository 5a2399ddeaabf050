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


def _allreduce_rank(rank, world, port, out):
    import torch.distributed as dist
    os.environ.update(MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port))
    dist.init_process_group("gloo", rank=rank, world_size=world)
    import bench
    out.put((rank, bench.allreduce([1.0 + rank, 5.0 - rank], [10 + rank, 2.5], world)))
    dist.destroy_process_group()


def test_two_gloo_ranks_allreduce_e2e_figures():
    """The end-to-end figures reduce like the device ones: maxima of the
    ranks' call times, sums of their solved queries and copied bytes."""
    pytest.importorskip("torch")
    import torch.multiprocessing as mp
    ctx = mp.get_context("spawn")
    q = ctx.Queue()
    port = _free_port()
    procs = [ctx.Process(target=_allreduce_rank, args=(r, 2, port, q)) for r in range(2)]
    for p in procs:
        p.start()
    got = [q.get(timeout=120) for _ in procs]
    for p in procs:
        p.join(timeout=60)
        assert p.exitcode == 0
    for _, (mx, sm) in got:
        assert mx == [2.0, 5.0] and sm == [21.0, 5.0]


def test_bench_gpus_flag_spawns_ranks():
    """`bench.py --gpus 2` without a launcher starts two ranks itself (here
    the CPU reference arm over gloo): rank 0 prints the one JSON line with
    n_gpus 2, the other rank exits without work."""
    import json
    import subprocess
    import sys
    from conftest import ROOT
    env = dict(os.environ)
    env.pop("WORLD_SIZE", None)
    r = subprocess.run([sys.executable, str(ROOT / "bench.py"), "--gpus", "2", "--impl", "reference",
                        "--workload", "panda_tabletop", "--queries", "8", "--steps", "1", "--warmup", "3"],
                       capture_output=True, text=True, timeout=600, env=env, cwd=str(ROOT))
    assert r.returncode == 0, r.stderr[-2000:]
    lines = [json.loads(x) for x in r.stdout.splitlines() if x.startswith("{")]
    assert len(lines) == 1 and lines[0]["impl"] == "reference" and lines[0]["n_gpus"] == 2
