"""The multi-rank path of bench.py (`--gpus N` under torchrun): independent chains per rank, the
whole-job rate over the slowest rank (max over ranks), every rank holding the same value. Two gloo
ranks on the CPU (no GPU)."""
import os
import socket
import sys

import pytest

torch = pytest.importorskip("torch")
import torch.distributed as dist  # noqa: E402
import torch.multiprocessing as mp  # noqa: E402

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def _free_port():
    s = socket.socket()
    s.bind(("127.0.0.1", 0))
    p = s.getsockname()[1]
    s.close()
    return p


def _rank(rank, world, port, out):
    sys.path.insert(0, ROOT)
    os.environ.update(MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port), RANK=str(rank), WORLD_SIZE=str(world))
    dist.init_process_group("gloo", init_method="env://", rank=rank, world_size=world)
    import bench
    rate, secs = bench.job_rate(dist, world, 3, 1.0 + rank)   # rank 1 is the slower one
    out.put((rank, rate, secs))
    dist.destroy_process_group()


def test_job_rate_two_gloo_ranks():
    ctx = mp.get_context("spawn")
    q = ctx.Queue()
    port = _free_port()
    ps = [ctx.Process(target=_rank, args=(r, 2, port, q)) for r in range(2)]
    for p in ps:
        p.start()
    res = sorted(q.get(timeout=120) for _ in ps)
    for p in ps:
        p.join(timeout=60)
        assert p.exitcode == 0
    assert [r for r, _, _ in res] == [0, 1]
    for _, rate, secs in res:
        assert secs == 2.0 and rate == pytest.approx(2 * 3 / 2.0)


def test_job_rate_one_rank():
    sys.path.insert(0, ROOT)
    import bench
    assert bench.job_rate(None, 1, 4, 2.0) == (2.0, 2.0)
