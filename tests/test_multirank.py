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
