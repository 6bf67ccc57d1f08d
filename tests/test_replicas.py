"""The multi-GPU form of this path is N independent replicas (the fit does not
shard; each rank runs its own embedding on its own GPU). This checks, on CPU
with gloo and world_size 2, the host-side logic bench.py uses for it: the
barrier and the max over ranks of the timed region, and the whole-job value."""
import os
import socket

import pytest


def _free_port():
    s = socket.socket()
    s.bind(("127.0.0.1", 0))
    port = s.getsockname()[1]
    s.close()
    return port


def _worker(rank, world, port, out):
    os.environ.update(MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port), WORLD_SIZE=str(world), RANK=str(rank),
                      LOCAL_RANK=str(rank))
    import torch.distributed as dist

    import bench
    # each replica reports its own timed-region length; rank 1 is the slower one
    ms = 100.0 + 50.0 * rank
    worst = bench.barrier_and_max(ms, world)
    steps = 10
    value = world * steps / (worst / 1e3)
    out.put((rank, worst, value))
    dist.destroy_process_group()


def test_replica_max_over_ranks_gloo():
    import torch.multiprocessing as mp
    ctx = mp.get_context("spawn")
    q = ctx.Queue()
    port = _free_port()
    procs = [ctx.Process(target=_worker, args=(r, 2, port, q)) for r in range(2)]
    for p in procs:
        p.start()
    for p in procs:
        p.join(timeout=120)
        assert p.exitcode == 0
    res = sorted(q.get(timeout=10) for _ in range(2))
    assert [r[1] for r in res] == [150.0, 150.0]
    assert res[0][2] == pytest.approx(2 * 10 / 0.150)


def test_dist_info_defaults(monkeypatch):
    import bench
    for k in ("WORLD_SIZE", "RANK", "LOCAL_RANK"):
        monkeypatch.delenv(k, raising=False)
    assert bench.dist_info() == (1, 0, 0)
    assert bench.barrier_and_max(3.5, 1) == 3.5
