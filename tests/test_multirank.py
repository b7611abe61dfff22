"""CPU, world_size 2 over gloo: the multi-GPU form of the benchmark is
independent replicas (systems are independent; there is no exchange on the
data path).  Each rank solves its own starts, and the job's time is the max
over ranks.  This checks the two pieces of host logic that form relies on:
the per-rank seeds never collide, and the time reduction returns the slowest
rank's time on every rank."""
import os
import sys
from pathlib import Path

import pytest

ROOT = Path(__file__).resolve().parent.parent


def _rank_main(rank, world, port, out_dir):
    os.environ.update(MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port), RANK=str(rank),
                      WORLD_SIZE=str(world), LOCAL_RANK=str(rank))
    sys.path[:0] = [str(ROOT), str(ROOT / "dpcuda-v2_gb300")]
    import torch.distributed as dist
    import bench
    dist.init_process_group("gloo", rank=rank, world_size=world)
    seeds = [sd for k in range(12) for sd in bench.step_seeds(rank, k)]
    slowest = bench.reduce_max(10.0 + rank, device="cpu")
    gathered = [None] * world
    dist.all_gather_object(gathered, seeds)
    if rank == 0:
        flat = [sd for g in gathered for sd in g]
        ok = len(flat) == len(set(flat))
        Path(out_dir, "result.txt").write_text(f"{ok} {slowest}")
    else:
        Path(out_dir, f"slow{rank}.txt").write_text(str(slowest))
    dist.barrier()
    dist.destroy_process_group()


def test_replica_seeds_disjoint_and_time_is_max_over_ranks(tmp_path):
    torch = pytest.importorskip("torch")
    import socket
    with socket.socket() as sk:
        sk.bind(("127.0.0.1", 0))
        port = sk.getsockname()[1]
    torch.multiprocessing.spawn(_rank_main, args=(2, port, str(tmp_path)), nprocs=2, join=True)
    ok, slowest = (tmp_path / "result.txt").read_text().split()
    assert ok == "True"
    assert float(slowest) == 11.0
    assert float((tmp_path / "slow1.txt").read_text()) == 11.0


def test_reduce_max_without_process_group_is_identity():
    sys.path[:0] = [str(ROOT)]
    import bench
    assert bench.reduce_max(3.5) == 3.5


def test_partition_balances_uneven_systems():
    sys.path[:0] = [str(ROOT / "dpcuda-v2_gb300")]
    import numpy as np
    from dpcuda_gb300.ensemble import partition_systems
    rng = np.random.default_rng(3)
    n = np.floor(np.exp(rng.uniform(np.log(64), np.log(4096), 256))).astype(int)
    for world in (1, 2, 3, 8):
        parts = partition_systems(n, world)
        flat = sorted(k for p in parts for k in p)
        assert flat == list(range(len(n)))
        loads = [int(n[p].sum()) for p in parts]
        assert max(loads) - min(loads) <= n.max()


def _partition_rank(rank, world, port, out_dir):
    os.environ.update(MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port), RANK=str(rank),
                      WORLD_SIZE=str(world), LOCAL_RANK=str(rank))
    sys.path[:0] = [str(ROOT), str(ROOT / "dpcuda-v2_gb300")]
    import torch.distributed as dist
    from dpcuda_gb300.ensemble import partition_systems
    dist.init_process_group("gloo", rank=rank, world_size=world)
    sizes = [64, 4096, 700, 1500, 90, 2048, 333, 128, 1000]
    mine = partition_systems(sizes, world)[rank]
    gathered = [None] * world
    dist.all_gather_object(gathered, mine)
    if rank == 0:
        flat = sorted(k for g in gathered for k in g)
        Path(out_dir, "parts.txt").write_text(f"{flat == list(range(len(sizes)))} {gathered}")
    dist.barrier()
    dist.destroy_process_group()


def test_partition_is_consistent_across_ranks(tmp_path):
    """Every rank computes the same assignment on its own; together the ranks
    cover each system exactly once."""
    torch = pytest.importorskip("torch")
    import socket
    with socket.socket() as sk:
        sk.bind(("127.0.0.1", 0))
        port = sk.getsockname()[1]
    torch.multiprocessing.spawn(_partition_rank, args=(2, port, str(tmp_path)), nprocs=2, join=True)
    assert (tmp_path / "parts.txt").read_text().startswith("True")
