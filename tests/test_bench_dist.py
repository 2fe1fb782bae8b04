"""The multi-process path of bench.py (replicas, one rank per GPU), on the CPU
with two gloo ranks: the only collective is the max / sum of per-rank numbers,
whole-job throughput counts every rank's units against the slowest rank's
time, and ranks other than 0 of the reference arm exit without work."""
import io
import os
import socket
import sys
from contextlib import redirect_stdout

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def _free_port():
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def _rank(rank, world, port, out):
    import torch.distributed as dist
    os.environ.update(MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port), RANK=str(rank), WORLD_SIZE=str(world),
                      LOCAL_RANK=str(rank))
    sys.path.insert(0, ROOT)
    import bench
    dist.init_process_group("gloo", rank=rank, world_size=world)
    try:
        mx = bench.reduce_over_ranks(10.0 + rank, "max")
        sm = bench.reduce_over_ranks(100.0 * (rank + 1), "sum")
        rate = bench.whole_job_rate(512, mx, world)
        # the reference arm: rank 0 alone measures; the others return at once
        buf = io.StringIO()
        ran = True
        if rank != 0:
            class A:
                steps, warmup = 1, 1
            with redirect_stdout(buf):
                ran = bench.run_reference(A()) is not None
        out.put((rank, mx, sm, rate, ran, buf.getvalue()))
    finally:
        dist.destroy_process_group()


def test_two_gloo_ranks():
    torch = pytest.importorskip("torch")
    import torch.multiprocessing as mp
    ctx = mp.get_context("spawn")
    q = ctx.Queue()
    port = _free_port()
    procs = [ctx.Process(target=_rank, args=(r, 2, port, q)) for r in range(2)]
    for p in procs:
        p.start()
    res = sorted(q.get(timeout=120) for _ in procs)
    for p in procs:
        p.join(timeout=60)
        assert p.exitcode == 0
    for rank, mx, sm, rate, ran, printed in res:
        assert mx == 11.0 and sm == 300.0
        assert abs(rate - 2 * 512 / 11e-3) < 1e-6
        if rank == 1:
            assert not ran and printed == ""


def test_single_process_is_identity():
    sys.path.insert(0, ROOT)
    import bench
    assert bench.reduce_over_ranks(3.5) == 3.5
    assert bench.whole_job_rate(1, 4.0, 1) == 250.0
