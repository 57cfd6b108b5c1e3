"""bench.py's multi-rank path on the CPU: two gloo ranks, each an independent
replica; the reported time is the slowest rank's (max over ranks) and only
rank 0 prints."""
import os
import socket
import sys

import torch.multiprocessing as mp

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def _free_port():
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def _worker(rank, world, port, out):
    import torch.distributed as dist
    sys.path.insert(0, ROOT)
    os.environ.update(MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port))
    dist.init_process_group("gloo", rank=rank, world_size=world)
    import bench
    t = bench.max_over_ranks(1.0 + rank, world, "cpu")
    out[rank] = t
    dist.barrier()
    dist.destroy_process_group()


def test_max_over_ranks_gloo():
    world = 2
    port = _free_port()
    mgr = mp.get_context("spawn").Manager()
    out = mgr.dict()
    mp.start_processes(_worker, args=(world, port, out), nprocs=world, start_method="spawn", join=True)
    assert dict(out) == {0: 2.0, 1: 2.0}


def test_reference_arm_only_rank0_prints(monkeypatch, capsys):
    sys.path.insert(0, ROOT)
    import bench
    monkeypatch.setenv("RANK", "1")
    monkeypatch.setenv("WORLD_SIZE", "2")
    monkeypatch.setattr(sys, "argv", ["bench.py", "--impl", "reference"])
    assert bench.main() == 0
    assert capsys.readouterr().out == ""


def _shard_worker(rank, world, port, out):
    import torch.distributed as dist
    sys.path.insert(0, ROOT)
    os.environ.update(MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port))
    dist.init_process_group("gloo", rank=rank, world_size=world)
    from pv2013_gb300.shard import shard
    weights = [(7919 * (i + 3)) % 1009 + 50 for i in range(64)]      # uneven vessel sizes
    mine = shard(weights, rank, world)
    got = [None] * world
    dist.all_gather_object(got, mine)
    out[rank] = got
    dist.destroy_process_group()


def test_ensemble_shards_are_disjoint_complete_and_balanced():
    """Two gloo ranks compute the partition of 64 uneven instances on their
    own: the ranks agree, every instance is on exactly one rank, and the
    loads differ by at most the heaviest instance."""
    world = 2
    port = _free_port()
    mgr = mp.get_context("spawn").Manager()
    out = mgr.dict()
    mp.start_processes(_shard_worker, args=(world, port, out), nprocs=world, start_method="spawn", join=True)
    a, b = out[0], out[1]
    assert a == b
    flat = sorted(i for part in a for i in part)
    assert flat == list(range(64))
    weights = [(7919 * (i + 3)) % 1009 + 50 for i in range(64)]
    loads = [sum(weights[i] for i in part) for part in a]
    assert abs(loads[0] - loads[1]) <= max(weights)


def test_partition_edge_cases():
    sys.path.insert(0, ROOT)
    from pv2013_gb300.shard import partition
    assert partition([5, 1, 1], 1) == [[0, 1, 2]]
    assert partition([5, 1, 1], 4) == [[0], [1], [2], []]
    assert partition([], 2) == [[], []]
