"""The N > 1 bench path on CPU: two gloo ranks (127.0.0.1) aggregate their
timed regions as the slowest replica and report whole-job throughput; the
replicas share nothing else (each builds and runs its own circuits)."""
import os
import socket

import pytest
import torch.distributed as dist
import torch.multiprocessing as mp


def _free_port():
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def _worker(rank, ws, port, out):
    os.environ.update(MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port), RANK=str(rank), WORLD_SIZE=str(ws),
                      LOCAL_RANK=str(rank))
    import bench

    dist.init_process_group("gloo", rank=rank, world_size=ws)
    try:
        seconds = [1.5, 2.5][rank]
        slow = bench.max_over_ranks(seconds, ws, "cpu")
        value = bench.replica_value(100.0, ws, slow)
        got_ws, got_rank, got_local = bench.dist_info()
        out.put((rank, slow, value, got_ws, got_rank, got_local))
    finally:
        dist.destroy_process_group()


def test_two_rank_max_and_weak_scaling():
    ctx = mp.get_context("spawn")
    q = ctx.Queue()
    port = _free_port()
    procs = [ctx.Process(target=_worker, args=(r, 2, port, q)) for r in range(2)]
    for p in procs:
        p.start()
    for p in procs:
        p.join(120)
        assert p.exitcode == 0
    res = sorted(q.get(timeout=10) for _ in range(2))
    for rank, slow, value, ws, got_rank, local in res:
        assert slow == pytest.approx(2.5) and value == pytest.approx(2 * 100.0 / 2.5)
        assert ws == 2 and got_rank == rank and local == rank


def test_single_rank_passthrough():
    import bench

    assert bench.max_over_ranks(3.0, 1, "cpu") == 3.0
    assert bench.replica_value(10.0, 1, 2.0) == 5.0
