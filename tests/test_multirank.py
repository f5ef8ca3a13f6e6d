"""The bench's replica path for N > 1 GPUs, on CPU: two gloo ranks run the timing reductions
(max of the step times, sum of the work), and the batched workload's instances are split across
ranks without overlap and with balanced work.  No GPU."""
import os
import socket

import pytest

torch = pytest.importorskip("torch")

import bench  # noqa: E402


def _free_port():
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def _rank_main(rank, world, port, out):
    os.environ.update(MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port), RANK=str(rank), WORLD_SIZE=str(world))
    torch.distributed.init_process_group("gloo", rank=rank, world_size=world)
    try:
        bench._barrier(world, cuda=False)
        ms = bench._max_over_ranks(10.0 + 5.0 * rank, world, "cpu")
        work = bench._sum_over_ranks(100.0 * (rank + 1), world, "cpu")
        out.put((rank, ms, work))
    finally:
        torch.distributed.destroy_process_group()


def test_two_gloo_ranks_reduce_timing_and_work():
    ctx = torch.multiprocessing.get_context("spawn")
    q = ctx.Queue()
    port = _free_port()
    procs = [ctx.Process(target=_rank_main, args=(r, 2, port, q)) for r in range(2)]
    for p in procs:
        p.start()
    for p in procs:
        p.join(120)
    assert all(p.exitcode == 0 for p in procs)
    got = sorted(q.get(timeout=10) for _ in range(2))
    assert got == [(0, 15.0, 300.0), (1, 15.0, 300.0)]   # every rank sees the max time and the total work


def test_partition_covers_every_instance_once_and_balances():
    import numpy as np

    rng = np.random.default_rng(4)
    ns = rng.integers(10, 23, size=512)
    ks = rng.choice([1, 4, 16], size=512)
    costs = [int(k) * (2 * int(n) + 1) * (1 << int(n)) for n, k in zip(ns, ks)]
    for world in (1, 2, 4, 8):
        parts = bench.partition_instances(costs, world)
        flat = sorted(i for p in parts for i in p)
        assert flat == list(range(512))
        loads = [sum(costs[i] for i in p) for p in parts]
        # largest-first greedy: no rank exceeds the mean by more than the largest instance
        assert max(loads) <= sum(costs) / world + max(costs)
    assert bench.partition_instances([5, 5], 2) == [[0], [1]]
    assert bench.partition_instances([], 3) == [[], [], []]
