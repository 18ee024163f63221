"""Multi-process (replicas-only) aggregation of bench.py on the CPU: two
gloo ranks, different per-rank times -> every rank sees the slowest; rank 0's
form decision reaches every rank.  No GPU."""
import os
import socket
import sys

import pytest
import torch
import torch.distributed as dist
import torch.multiprocessing as mp

REPO = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def _free_port():
    s = socket.socket()
    s.bind(("127.0.0.1", 0))
    p = s.getsockname()[1]
    s.close()
    return p


def _worker(rank, ws, port, q):
    sys.path.insert(0, REPO)
    os.environ.update(MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port))
    dist.init_process_group("gloo", rank=rank, world_size=ws)
    import bench
    tot = bench.replica_total_ms(10.0 + 5.0 * rank, dist)
    chosen = bench.agree("mixed" if rank == 0 else "plain", dist)
    q.put((rank, tot, chosen))
    dist.destroy_process_group()


@pytest.mark.parametrize("ws", [2])
def test_replica_aggregation(ws):
    ctx = mp.get_context("spawn")
    q = ctx.Queue()
    port = _free_port()
    procs = [ctx.Process(target=_worker, args=(r, ws, port, q)) for r in range(ws)]
    for p in procs:
        p.start()
    out = [q.get(timeout=120) for _ in range(ws)]
    for p in procs:
        p.join(timeout=60)
        assert p.exitcode == 0
    for rank, tot, chosen in out:
        assert tot == 10.0 + 5.0 * (ws - 1)
        assert chosen == "mixed"
