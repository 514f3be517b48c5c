"""The multi-GPU path is replicas only: every rank solves its own instance and
bench.py reports the units of all ranks over the slowest rank's time.  The
aggregation runs here as world-size-2 gloo ranks on the CPU."""
import os
import socket

import pytest
import torch.multiprocessing as mp


def _free_port():
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def _rank(rank, world, port, out):
    import torch.distributed as dist
    import bench
    os.environ.update(MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port))
    dist.init_process_group("gloo", rank=rank, world_size=world)
    try:
        ms = [200.0, 250.0][rank]
        units = [30, 20][rank]
        out[rank] = bench.replica_throughput(ms, units, world, "cpu")
    finally:
        dist.destroy_process_group()


def test_replica_throughput_two_gloo_ranks():
    ctx = mp.get_context("spawn")
    with ctx.Manager() as m:
        out = m.dict()
        port = _free_port()
        procs = [ctx.Process(target=_rank, args=(r, 2, port, out)) for r in range(2)]
        for p in procs:
            p.start()
        for p in procs:
            p.join(120)
            assert p.exitcode == 0
        res = dict(out)
    for r in range(2):
        ms_max, value = res[r]
        assert ms_max == 250.0
        assert value == pytest.approx(50 / 0.25)


def test_replica_throughput_single_rank():
    import bench
    assert bench.replica_throughput(100.0, 10, 1, "cpu") == (100.0, pytest.approx(100.0))
