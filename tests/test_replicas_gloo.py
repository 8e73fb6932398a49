"""The replica reduction used by bench.py --gpus N, on world-size-2 gloo CPU ranks."""
import os
import sys

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def _worker(rank, port, q):
    sys.path.insert(0, ROOT)
    os.environ.update({"RANK": str(rank), "LOCAL_RANK": str(rank), "WORLD_SIZE": "2",
                       "MASTER_ADDR": "127.0.0.1", "MASTER_PORT": str(port)})
    from fluidloom_gb300.replicas import Replicas
    r = Replicas(backend="gloo")
    r.barrier()
    ms = r.max(10.0 + rank)          # slowest rank's time
    lups = r.sum(1000.0 * (rank + 1))  # all ranks' updates
    q.put((rank, ms, lups))
    r.close()


def test_replica_reduction_two_ranks():
    torch = pytest.importorskip("torch")
    import torch.multiprocessing as mp
    import socket
    s = socket.socket()
    s.bind(("127.0.0.1", 0))
    port = s.getsockname()[1]
    s.close()
    ctx = mp.get_context("spawn")
    q = ctx.Queue()
    ps = [ctx.Process(target=_worker, args=(r, port, q)) for r in range(2)]
    for p in ps:
        p.start()
    for p in ps:
        p.join(120)
        assert p.exitcode == 0
    res = sorted(q.get(timeout=10) for _ in range(2))
    assert all(ms == 11.0 and lups == 3000.0 for _, ms, lups in res)


def test_single_rank_is_identity():
    from fluidloom_gb300.replicas import Replicas
    os.environ.pop("WORLD_SIZE", None)
    r = Replicas()
    assert r.world == 1 and r.max(3.5) == 3.5 and r.sum(2.0) == 2.0
