"""Multi-GPU form of the bench: independent replicas, one per rank, combined on the
host by the slowest rank's time.  Exercised here with two gloo ranks on the CPU."""
import os
import socket

import pytest

from conftest import ROOT


def _free_port():
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def _rank_main(rank, world, port, out):
    import sys
    sys.path.insert(0, ROOT)
    import torch.distributed as dist
    import bench
    os.environ.update(MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port))
    dist.init_process_group("gloo", rank=rank, world_size=world)
    local = [1.5, 2.5][rank]  # each replica's own time for its steps
    slow = bench.slowest_rank(local, world)
    out[rank] = (slow, bench.job_mpoints_per_s(10_000_000, 4, world, slow))
    dist.destroy_process_group()


def test_replicas_take_the_slowest_rank():
    torch = pytest.importorskip("torch")
    mp = torch.multiprocessing.get_context("spawn")
    with mp.Manager() as m:
        out = m.dict()
        port = _free_port()
        procs = [mp.Process(target=_rank_main, args=(r, 2, port, out)) for r in range(2)]
        for p in procs:
            p.start()
        for p in procs:
            p.join(120)
            assert p.exitcode == 0
        res = dict(out)
    for r in range(2):
        slow, value = res[r]
        assert slow == 2.5
        assert value == pytest.approx(2 * 10_000_000 * 4 / 2.5 / 1e6)


def test_single_rank_is_identity():
    import sys
    sys.path.insert(0, ROOT)
    import bench
    assert bench.slowest_rank(3.0, 1) == 3.0
    assert bench.job_mpoints_per_s(1_000_000, 2, 1, 0.5) == pytest.approx(4.0)
