"""The replica path of bench.py on two gloo ranks (CPU, 127.0.0.1): the
job's step time is the slowest rank's and its band voxels the sum over
ranks; the reference arm runs on rank 0 only."""
import io
import os
import socket
import sys
from contextlib import redirect_stdout

import pytest

torch = pytest.importorskip("torch")


def _free_port():
    s = socket.socket()
    s.bind(("127.0.0.1", 0))
    port = s.getsockname()[1]
    s.close()
    return port


def _worker(rank, world, port, q):
    import torch.distributed as dist
    os.environ.update(MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port), RANK=str(rank), WORLD_SIZE=str(world),
                      LOCAL_RANK=str(rank))
    dist.init_process_group("gloo", rank=rank, world_size=world)
    import bench
    q.put((rank, bench.combine_ranks(10.0 + rank, 100 * (rank + 1), world, "cpu")))
    dist.barrier()
    dist.destroy_process_group()


def test_combine_ranks_two_gloo_ranks():
    import torch.multiprocessing as mp
    ctx = mp.get_context("spawn")
    q = ctx.Queue()
    port = _free_port()
    procs = [ctx.Process(target=_worker, args=(r, 2, port, q)) for r in range(2)]
    for p in procs:
        p.start()
    for p in procs:
        p.join(timeout=180)
    assert all(p.exitcode == 0 for p in procs)
    got = dict(q.get(timeout=10) for _ in range(2))
    assert got[0] == got[1] == (11.0, 300)


def test_single_rank_passthrough():
    import bench
    assert bench.combine_ranks(12.5, 7, 1) == (12.5, 7)


def test_reference_arm_only_on_rank_zero(monkeypatch):
    import bench
    monkeypatch.setenv("RANK", "1")
    monkeypatch.setenv("WORLD_SIZE", "2")

    class A:
        steps, warmup, gpus = 1, 1, 2

    buf = io.StringIO()
    with redirect_stdout(buf):
        assert bench.run_reference(A()) is None
    assert buf.getvalue() == ""
