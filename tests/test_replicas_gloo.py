"""bench.py --gpus N runs N independent replicas (the solve does not shard):
each rank times its own copy of the workload, the timed region is the maximum
over the ranks (all_reduce MAX over gloo), and the whole-job value counts every
rank's solves.  Two gloo ranks on the CPU check that aggregation, and that the
reference arm does its work on rank 0 only."""
import os
import socket
import sys

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
sys.path.insert(0, ROOT)


def _free_port():
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def _rank(rank, world, port, out):
    import torch.distributed as dist

    import bench
    os.environ.update({"MASTER_ADDR": "127.0.0.1", "MASTER_PORT": str(port), "RANK": str(rank),
                       "WORLD_SIZE": str(world), "LOCAL_RANK": str(rank)})
    dist.init_process_group("gloo", rank=rank, world_size=world)
    ws, r, local = bench.dist_env()
    local_ms = 100.0 * (rank + 1)  # the slower rank sets the timed region
    total = bench.replica_time_ms(local_ms, dist)
    dist.barrier()
    dist.destroy_process_group()
    out.put((r, ws, local, total, bench.replica_value(ws, 4, total)))


def test_replica_timing_is_the_max_over_two_gloo_ranks():
    torch = pytest.importorskip("torch")
    mp = torch.multiprocessing.get_context("spawn")
    q = mp.Queue()
    port = _free_port()
    procs = [mp.Process(target=_rank, args=(k, 2, port, q)) for k in range(2)]
    for p in procs:
        p.start()
    res = sorted(q.get(timeout=120) for _ in procs)
    for p in procs:
        p.join(timeout=60)
        assert p.exitcode == 0
    for k, (rank, ws, local, total, value) in enumerate(res):
        assert rank == k and local == k and ws == 2
        assert total == 200.0  # max over ranks, seen by both
        assert value == pytest.approx(2 * 4 / 0.2)  # 8 solves of all ranks in 0.2 s


def test_single_process_needs_no_collective():
    import bench
    assert bench.replica_time_ms(123.0) == 123.0
    assert bench.replica_value(1, 8, 1000.0) == pytest.approx(8.0)


def test_reference_arm_runs_on_rank_0_only(monkeypatch):
    import bench
    monkeypatch.setenv("WORLD_SIZE", "2")
    monkeypatch.setenv("RANK", "1")
    # a non-zero rank returns before touching the oracle or the workload
    assert bench.run_reference(None) is None
