"""bench.py's replica mode (`--gpus N` under torchrun): N independent blends,
no data-path collective; the job's time is the slowest rank's (an all-reduce
MAX) and the throughput counts every rank's units.  Checked with two gloo
ranks on the CPU."""
import os
import socket

import pytest

torch = pytest.importorskip("torch")


def _free_port() -> int:
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def _rank(rank, ws, port, q):
    os.environ.update(MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port), RANK=str(rank), WORLD_SIZE=str(ws),
                      LOCAL_RANK=str(rank))
    import torch.distributed as dist
    import bench
    dist.init_process_group("gloo", rank=rank, world_size=ws)
    try:
        ws_, rank_, local_ = bench.dist_setup()
        ms = bench.max_over_ranks(10.0 + 5.0 * rank, ws_, device="cpu")
        q.put((rank_, local_, ms, bench.replica_value(25.17, ws_, 4, ms)))
    finally:
        dist.destroy_process_group()


def test_two_replicas_take_the_slowest_rank():
    import multiprocessing as mp
    ctx = mp.get_context("spawn")
    q = ctx.Queue()
    port = _free_port()
    procs = [ctx.Process(target=_rank, args=(r, 2, port, q)) for r in range(2)]
    for p in procs:
        p.start()
    for p in procs:
        p.join(120)
        assert p.exitcode == 0
    got = sorted(q.get(timeout=10) for _ in procs)
    assert [g[0] for g in got] == [0, 1] and [g[1] for g in got] == [0, 1]
    for _, _, ms, value in got:
        assert ms == 15.0                                  # the slower rank's time on every rank
        assert value == pytest.approx(2 * 25.17 * 4 / 0.015)


def test_single_rank_is_its_own_time():
    import bench
    assert bench.max_over_ranks(12.5, 1) == 12.5
    assert bench.replica_value(25.17, 1, 10, 12.5) == pytest.approx(25.17 * 10 / 0.0125)
