"""The replica path of bench.py with two ranks (gloo on CPU): the whole-job figures are the
slowest rank's timed region and the sum of the ranks' particles, so value = total
particles x steps / max time."""
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
    os.environ.update(MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port))
    dist.init_process_group("gloo", rank=rank, world_size=world)
    import bench
    ms, n = bench.rank_totals(10.0 + 5.0 * rank, 1000 + rank, dist, "cpu")
    out.put((rank, ms, n))
    dist.destroy_process_group()


def test_rank_totals_two_gloo_ranks():
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
    assert res == [(0, 15.0, 2001), (1, 15.0, 2001)]


def test_rank_totals_single_process():
    import bench
    assert bench.rank_totals(12.5, 7, None, "cpu") == (12.5, 7)
