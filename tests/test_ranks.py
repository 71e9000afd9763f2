"""The replicated (N > 1) bench path on CPU: two gloo ranks, whole-job units summed and the
slowest rank's time taken, as bench.py reports them."""
import os
import socket
import sys

import pytest

ROOT = os.path.abspath(os.path.join(os.path.dirname(__file__), ".."))


def _free_port():
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def _rank(rank, world, port, out):
    sys.path.insert(0, ROOT)
    import torch.distributed as dist
    os.environ.update(MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port))
    dist.init_process_group("gloo", rank=rank, world_size=world)
    import bench
    units, seconds = bench.combine_ranks(1000.0 * (rank + 1), 0.5 + rank, world)
    out.put((rank, units, seconds))
    dist.barrier()
    dist.destroy_process_group()


def test_combine_ranks_two_gloo_ranks():
    torch = pytest.importorskip("torch")
    import torch.multiprocessing as mp
    ctx = mp.get_context("spawn")
    q = ctx.Queue()
    port = _free_port()
    procs = [ctx.Process(target=_rank, args=(r, 2, port, q)) for r in range(2)]
    for p in procs:
        p.start()
    got = sorted(q.get(timeout=120) for _ in range(2))
    for p in procs:
        p.join(timeout=60)
        assert p.exitcode == 0
    assert [g[1:] for g in got] == [(3000.0, 1.5), (3000.0, 1.5)]


def test_combine_ranks_single_process():
    sys.path.insert(0, ROOT)
    import bench
    assert bench.combine_ranks(123.0, 2.0, 1) == (123.0, 2.0)
