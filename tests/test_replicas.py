"""Replica aggregation of bench.py on CPU: two gloo ranks, each timing its
own work.  The job's time is the slowest rank's, its throughput all ranks'
units over that time; the reference arm does its work on rank 0 only."""
import os
import socket
import sys
import types

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def _free_port():
    s = socket.socket()
    s.bind(("127.0.0.1", 0))
    port = s.getsockname()[1]
    s.close()
    return port


def _rank(rank, world, port, q):
    os.environ.update(MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port), RANK=str(rank),
                      WORLD_SIZE=str(world), LOCAL_RANK=str(rank))
    sys.path.insert(0, ROOT)
    import torch.distributed as dist
    import bench
    dist.init_process_group("gloo", rank=rank, world_size=world)
    try:
        secs = 1.5 + rank  # rank 1 is the slow one
        worst = bench.max_over_ranks(secs)
        value = bench.replica_value(10, world, worst)
        # the reference arm: ranks other than 0 return without work
        ran = bench.run_reference(types.SimpleNamespace(workload="large_cut")) if rank else "skip"
        q.put((rank, worst, value, ran))
    finally:
        dist.destroy_process_group()


def test_two_gloo_replicas():
    torch = pytest.importorskip("torch")
    mp = torch.multiprocessing.get_context("spawn")
    q = mp.Queue()
    port = _free_port()
    ps = [mp.Process(target=_rank, args=(r, 2, port, q)) for r in range(2)]
    for p in ps:
        p.start()
    out = sorted(q.get(timeout=120) for _ in ps)
    for p in ps:
        p.join(timeout=60)
        assert p.exitcode == 0
    for rank, worst, value, ran in out:
        assert worst == 2.5                    # max over ranks
        assert abs(value - 2 * 10 / 2.5) < 1e-12
    assert out[1][3] is None                   # rank 1 of the reference arm: no work


def test_single_process_is_its_own_max():
    sys.path.insert(0, ROOT)
    import bench
    assert bench.max_over_ranks(3.25) == 3.25
    assert bench.replica_value(7, 1, 2.0) == 3.5


def test_run_split_spreads_steps_and_overlaps_blocking_calls():
    """bench.run_split: `steps` calls spread round robin over the handles'
    threads, the threads overlapping calls that block outside the
    interpreter (as the engine's C calls do), and an error in one thread
    raised on the caller."""
    import time
    sys.path.insert(0, ROOT)
    import bench
    calls = [0, 0, 0]

    def make(j):
        def step():
            calls[j] += 1
            time.sleep(0.02)
            return j
        return step

    t0 = time.perf_counter()
    assert bench.run_split([make(0), make(1), make(2)], 10) == 0
    wall = time.perf_counter() - t0
    assert calls == [4, 3, 3]
    assert wall < 0.15   # 4 sleeps of 20 ms in sequence at most, not 10

    def bad():
        raise RuntimeError("engine error")

    with pytest.raises(RuntimeError, match="engine error"):
        bench.run_split([make(0), bad], 6)
