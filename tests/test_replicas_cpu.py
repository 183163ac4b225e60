"""Multi-GPU runs place independent requests on the ranks (nothing is
exchanged): the bench's process-group logic -- the request shards, the
barrier, the max over ranks of the timed intervals and the sum of their work,
rank 0 alone reporting -- checked with two gloo ranks on the CPU."""
import os
import socket
import subprocess
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
    sys.path.insert(0, os.path.join(REPO, "ader-dg_gb300"))
    import bench
    d, r, w, lr = bench.dist_init(backend="gloo")
    assert (r, w, lr) == (rank, ws, rank)
    bench.barrier(d)
    # each rank times its own shard; the job's time is the slowest rank's and
    # its work the sum of the ranks'
    t = bench.allmax(d, 1.0 + 0.5 * rank)
    work = bench.allsum(d, 10.0 * (rank + 1))
    shard = [(s["name"], s["N"], s["side"], s["params"]) for s in bench.mix_specs(8, rank, ws)]
    out.put((rank, t, work, shard))
    d.destroy_process_group()


def test_two_ranks_shard_the_requests():
    ctx = mp.get_context("spawn")
    q = ctx.Queue()
    port = _free_port()
    procs = [ctx.Process(target=_rank, args=(r, 2, port, q)) for r in range(2)]
    for p in procs:
        p.start()
    for p in procs:
        p.join(120)
        assert p.exitcode == 0
    res = {r: (t, w, sh) for r, t, w, sh in (q.get(timeout=10) for _ in range(2))}
    assert res[0][:2] == res[1][:2] == (1.5, 30.0)
    # the shards are disjoint and together they are the first 16 requests of the mix
    sys.path.insert(0, os.path.join(REPO, "ader-dg_gb300"))
    import aderdg
    mix = [(s["name"], s["N"], s["side"], s["params"]) for s in aderdg.workloads.request_mix(1024, seed=0)[:16]]
    assert res[0][2] == mix[0::2] and res[1][2] == mix[1::2]
    assert len(res[0][2]) == len(res[1][2]) == 8


def test_gpus_flag_without_ranks_fails_loudly():
    """--gpus 2 without a launcher that starts two ranks is refused, not run as one GPU."""
    env = dict(os.environ)
    for k in ("WORLD_SIZE", "RANK", "LOCAL_RANK"):
        env.pop(k, None)
    r = subprocess.run([sys.executable, os.path.join(REPO, "bench.py"), "--gpus", "2", "--steps", "1"],
                       capture_output=True, text=True, env=env, timeout=120)
    assert r.returncode == 2 and "torchrun" in r.stderr
