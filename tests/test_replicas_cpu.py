"""Multi-GPU runs are replicas (requests are independent; nothing is
exchanged): the bench's process-group logic -- barrier, max over ranks of
the timed intervals, rank 0 alone reporting -- checked with two gloo ranks on
the CPU."""
import os
import socket
import sys

import pytest

torch = pytest.importorskip("torch")
import torch.distributed as dist  # noqa: E402
import torch.multiprocessing as mp  # noqa: E402

REPO = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def _free_port():
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def _rank(rank, ws, port, out):
    os.environ.update(RANK=str(rank), LOCAL_RANK=str(rank), WORLD_SIZE=str(ws), MASTER_ADDR="127.0.0.1",
                      MASTER_PORT=str(port))
    sys.path.insert(0, REPO)
    import bench
    d, r, w, lr = bench.dist_init(backend="gloo")
    assert (r, w, lr) == (rank, ws, rank)
    bench.barrier(d)
    # each rank times its own replica; the job's time is the slowest rank's
    t = bench.allmax(d, 1.0 + 0.5 * rank)
    out.put((rank, t))
    d.destroy_process_group()


def test_two_replicas_max_over_ranks():
    ctx = mp.get_context("spawn")
    q = ctx.Queue()
    port = _free_port()
    procs = [ctx.Process(target=_rank, args=(r, 2, port, q)) for r in range(2)]
    for p in procs:
        p.start()
    for p in procs:
        p.join(120)
        assert p.exitcode == 0
    res = dict(q.get(timeout=10) for _ in range(2))
    assert res == {0: 1.5, 1: 1.5}
