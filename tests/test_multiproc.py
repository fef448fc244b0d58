"""The multi-rank host logic of bench.py on CPU with gloo (world size 2): the job time
is the maximum over the ranks, the reference arm under torchrun prints one line from
rank 0 while the other rank exits cleanly, and the batched workload's problems are
split over the ranks (each problem on one rank, the work balanced, the totals summed).
(With more than one GPU, bench.py runs one replica of the assembly workload per rank
and splits the batch's problems between the ranks under this same logic.)"""
import json
import os
import socket
import subprocess
import sys

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def free_port():
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def _worker(rank, world, port, q):
    os.environ.update(MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port), RANK=str(rank), WORLD_SIZE=str(world))
    import torch.distributed as dist

    dist.init_process_group("gloo", rank=rank, world_size=world)
    sys.path.insert(0, ROOT)
    import bench

    q.put((rank, bench.max_over_ranks(1.5 * (rank + 1), world, "cpu")))
    dist.barrier()
    dist.destroy_process_group()


def test_max_over_ranks_gloo():
    import torch.multiprocessing as mp

    ctx = mp.get_context("spawn")
    q = ctx.Queue()
    port = free_port()
    procs = [ctx.Process(target=_worker, args=(r, 2, port, q)) for r in range(2)]
    for p in procs:
        p.start()
    got = dict(q.get(timeout=300) for _ in procs)
    for p in procs:
        p.join(timeout=300)
        assert p.exitcode == 0
    assert got == {0: 3.0, 1: 3.0}


def test_reference_arm_two_ranks():
    cmd = [sys.executable, "-m", "torch.distributed.run", "--nnodes=1", "--nproc-per-node", "2", "--master-addr",
           "127.0.0.1", "--master-port", str(free_port()), os.path.join(ROOT, "bench.py"), "--impl", "reference",
           "--gpus", "2", "--steps", "1", "--warmup", "1", "--cpu-n", "10"]
    r = subprocess.run(cmd, cwd=ROOT, capture_output=True, text=True, timeout=600)
    assert r.returncode == 0, r.stderr[-2000:]
    lines = [ln for ln in r.stdout.splitlines() if ln.startswith("{")]
    assert len(lines) == 1
    d = json.loads(lines[0])
    assert d["impl"] == "reference" and d["n_gpus"] == 2 and d["value"] > 0
    assert d["e2e"]["h2d_bytes_per_step"] == 0


@pytest.mark.parametrize("world", [1, 2, 3, 8])
def test_batch_shard_partition(world):
    """The batch split over ranks (proxpde_gb300.batch.shard): every problem on exactly
    one rank, and the ranks' work (nonzeros x n) within 10 % of each other for up to 8
    ranks on the 256-problem batch."""
    import numpy as np

    sys.path.insert(0, ROOT)
    from proxpde_gb300 import batch

    sizes = batch.problem_sizes()
    shards = [batch.shard(sizes, 128, r, world) for r in range(world)]
    allp = np.sort(np.concatenate(shards))
    assert np.array_equal(allp, np.arange(sizes.size))
    cost = np.where(np.arange(sizes.size) < 128, 27.0, 15.0) * (sizes + 1.0) ** 3 * sizes
    loads = np.array([cost[s].sum() for s in shards])
    assert loads.max() <= 1.1 * loads.mean()


def _shard_worker(rank, world, port, q):
    os.environ.update(MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port), RANK=str(rank), WORLD_SIZE=str(world))
    import torch
    import torch.distributed as dist

    dist.init_process_group("gloo", rank=rank, world_size=world)
    sys.path.insert(0, ROOT)
    from proxpde_gb300 import batch

    import bench

    mine = batch.shard(batch.problem_sizes(), 128, rank, world)
    got = [None] * world
    dist.all_gather_object(got, mine.tolist())
    # the job's element count: the sum over the ranks of their shards' elements
    elems = sum(int(n) ** 3 * (1 if p < 128 else 6) for p, n in zip(mine, batch.problem_sizes()[mine]))
    total = bench.job_sum(elems, world, "cpu")
    q.put((rank, got, total))
    dist.barrier()
    dist.destroy_process_group()


def test_batch_shard_gloo():
    """Two gloo ranks: each computes its shard of the batch; together they cover every
    problem once, and the job's element count is summed over the ranks."""
    import numpy as np
    import torch.multiprocessing as mp

    sys.path.insert(0, ROOT)
    from proxpde_gb300 import batch

    ctx = mp.get_context("spawn")
    q = ctx.Queue()
    port = free_port()
    procs = [ctx.Process(target=_shard_worker, args=(r, 2, port, q)) for r in range(2)]
    for p in procs:
        p.start()
    res = dict((r, (g, t)) for r, g, t in (q.get(timeout=300) for _ in procs))
    for p in procs:
        p.join(timeout=300)
        assert p.exitcode == 0
    (g0, t0), (g1, t1) = res[0], res[1]
    assert g0 == g1
    assert sorted(g0[0] + g0[1]) == list(range(256)) and not set(g0[0]) & set(g0[1])
    sizes = batch.problem_sizes()
    expect = sum(int(n) ** 3 * (1 if p < 128 else 6) for p, n in enumerate(sizes))
    assert t0 == t1 == expect
