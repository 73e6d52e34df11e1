"""Replicas on several GPUs (one independent 96^3 Newton solve per rank, no
collective on the data path): the host logic that turns per-rank times into the
job's rate, run as world-size-2 gloo ranks on the CPU."""
import os
import socket

import pytest

torch = pytest.importorskip("torch")
import torch.distributed as dist  # noqa: E402
import torch.multiprocessing as mp  # noqa: E402


def _free_port():
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def _rank(rank, world, port, out):
    os.environ.update(MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port), RANK=str(rank), WORLD_SIZE=str(world))
    dist.init_process_group("gloo", rank=rank, world_size=world)
    try:
        import bench
        local = [1.5, 2.25][rank]
        sec = bench.replica_seconds(local, device="cpu")
        out.put((rank, sec, bench.job_rate(world, 5, sec), bench.dist_env()))
    finally:
        dist.destroy_process_group()


def test_replica_time_is_the_slowest_rank_and_the_rate_counts_every_rank():
    ctx = mp.get_context("spawn")
    q = ctx.Queue()
    port = _free_port()
    procs = [ctx.Process(target=_rank, args=(r, 2, port, q)) for r in range(2)]
    for p in procs:
        p.start()
    got = sorted(q.get(timeout=120) for _ in procs)
    for p in procs:
        p.join(timeout=60)
        assert p.exitcode == 0
    for rank, sec, rate, env in got:
        assert sec == 2.25                       # max over ranks
        assert rate == pytest.approx(2 * 5 / 2.25)
        assert env == (2, rank)


def test_single_process_keeps_its_own_time():
    import bench
    assert bench.replica_seconds(3.0, device="cpu") == 3.0
    assert bench.job_rate(1, 5, 2.0) == 2.5
