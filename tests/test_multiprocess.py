"""Multi-rank host logic of bench.py --gpus N, on CPU with the gloo backend
and two processes: replicas of the single-matrix solve report the slowest
rank's time; the batched workload splits its problems over the ranks (greedy
balancing, no collective on the data path) and rank 0 gathers the results."""
import os
import socket
import sys

import numpy as np
import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def _free_port():
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def _rank_main(rank, world, port, out_dir):
    import torch.distributed as dist
    sys.path.insert(0, ROOT)
    os.environ.update(MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port), RANK=str(rank), WORLD_SIZE=str(world),
                      LOCAL_RANK=str(rank))
    dist.init_process_group("gloo", init_method="env://", rank=rank, world_size=world)
    import bench
    r, w, local = bench.dist_env()
    assert (r, w, local) == (rank, world, rank)
    ms = bench.max_over_ranks(10.0 + 5.0 * rank, world)
    dist.barrier()
    with open(os.path.join(out_dir, f"rank{rank}.txt"), "w") as f:
        f.write(repr(ms))
    dist.destroy_process_group()


def test_two_rank_gloo_max_over_ranks(tmp_path):
    torch = pytest.importorskip("torch")
    import torch.multiprocessing as mp
    port = _free_port()
    mp.spawn(_rank_main, args=(2, port, str(tmp_path)), nprocs=2, join=True)
    vals = [float(open(tmp_path / f"rank{r}.txt").read()) for r in range(2)]
    assert vals == [15.0, 15.0]


def test_single_rank_needs_no_process_group():
    sys.path.insert(0, ROOT)
    import bench
    assert bench.max_over_ranks(3.5, 1) == 3.5


def test_shard_problems_balances_and_covers():
    sys.path.insert(0, ROOT)
    import bench
    rng = np.random.default_rng(2)
    w = [float(7 * int(m) ** 3) ** 1.75 for m in rng.integers(16, 41, size=64)]
    for world in (1, 2, 3, 8):
        parts = bench.shard_problems(w, world)
        assert sorted(q for p in parts for q in p) == list(range(len(w)))
        loads = [sum(w[q] for q in p) for p in parts]
        # greedy heaviest-first: no rank exceeds the mean by more than the heaviest problem
        assert max(loads) <= sum(w) / world + max(w) + 1e-6
        assert parts == bench.shard_problems(w, world)  # deterministic


def _batch_rank(rank, world, port, out_dir):
    """The batch bench's host logic on gloo: shard, a stand-in solve per
    problem (no GPU), slowest-rank time, and rank 0's gather in problem order."""
    import time
    import torch.distributed as dist
    sys.path.insert(0, ROOT)
    os.environ.update(MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port), RANK=str(rank), WORLD_SIZE=str(world))
    dist.init_process_group("gloo", init_method="env://", rank=rank, world_size=world)
    import bench
    sizes = [16, 40, 23, 31, 18, 37, 25]
    parts = bench.shard_problems([float(s) ** 3 for s in sizes], world)
    t0 = time.perf_counter()
    local = [dict(info=0, neig=5, iter=10 * sizes[q]) for q in parts[rank]]
    dt = time.perf_counter() - t0 + (1.0 if rank == 1 else 0.0)
    slowest = bench.max_over_ranks(dt, world)
    gathered = bench.gather_to_root(local, world)
    if rank == 0:
        merged = bench.merge_shards(parts, gathered)
        with open(os.path.join(out_dir, "batch.txt"), "w") as f:
            f.write(repr(([r["iter"] for r in merged], slowest >= 1.0)))
    else:
        assert gathered is None
    dist.destroy_process_group()


def test_two_rank_batch_sharding_gather(tmp_path):
    pytest.importorskip("torch")
    import torch.multiprocessing as mp
    mp.spawn(_batch_rank, args=(2, _free_port(), str(tmp_path)), nprocs=2, join=True)
    iters, slow = eval(open(tmp_path / "batch.txt").read())
    assert iters == [10 * s for s in [16, 40, 23, 31, 18, 37, 25]] and slow
