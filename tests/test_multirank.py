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


def _oracle_fire(indices, sts):
    """CPU stand-in for a rank's GPU: each system minimised by the oracle."""
    from oracle.oracle import DiskOracle
    out = []
    for k in indices:
        st = sts[k]
        o = DiskOracle(len(st["r"]), st["box"])
        o.set_arrays(x=st["x"], y=st["y"], r=st["r"], m=st["m"])
        o.setup_neighbors(0, 1.7 / 1.4, 0.2, 8.0, 0.5)
        steps, _ = o.minimize_fire(0.1, 1e-2, 0.0, 0.0, 3000, 1e-10)
        out.append({"steps": int(steps), "avg_pe": o.total_pe() / len(st["r"]),
                    "max_force": o.max_force()})
        o.close()
    return out


SOLVE_SIZES = [64, 300, 150, 90, 200, 120, 64, 250]


def _solve_rank(rank, world, port, out_dir):
    os.environ.update(MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port), RANK=str(rank),
                      WORLD_SIZE=str(world), LOCAL_RANK=str(rank))
    sys.path[:0] = [str(ROOT), str(ROOT / "dpcuda-v2_gb300")]
    import json
    import torch.distributed as dist
    from dpcuda_gb300.ensemble import solve_partitioned
    from oracle.oracle import disk_packing
    dist.init_process_group("gloo", rank=rank, world_size=world)
    sts = [disk_packing(n, 0.86, 500 + k) for k, n in enumerate(SOLVE_SIZES)]
    res = solve_partitioned(SOLVE_SIZES, lambda idx: _oracle_fire(idx, sts))
    if rank == 0:
        Path(out_dir, "gathered.json").write_text(json.dumps(res))
    else:
        Path(out_dir, f"rank{rank}.json").write_text(json.dumps(res))
    dist.barrier()
    dist.destroy_process_group()


def test_partitioned_solve_gathers_the_single_rank_results(tmp_path):
    """Two ranks each solve their share of uneven systems (the oracle standing
    in for a rank's GPU); rank 0 gathers every system's result in input order,
    equal to one rank solving them all."""
    torch = pytest.importorskip("torch")
    import json
    import socket
    sys.path[:0] = [str(ROOT), str(ROOT / "dpcuda-v2_gb300")]
    from dpcuda_gb300.ensemble import solve_partitioned
    from oracle.oracle import disk_packing
    with socket.socket() as sk:
        sk.bind(("127.0.0.1", 0))
        port = sk.getsockname()[1]
    torch.multiprocessing.spawn(_solve_rank, args=(2, port, str(tmp_path)), nprocs=2, join=True)
    gathered = json.loads((tmp_path / "gathered.json").read_text())
    assert json.loads((tmp_path / "rank1.json").read_text()) is None
    sts = [disk_packing(n, 0.86, 500 + k) for k, n in enumerate(SOLVE_SIZES)]
    single = solve_partitioned(SOLVE_SIZES, lambda idx: _oracle_fire(idx, sts))
    assert gathered == single
