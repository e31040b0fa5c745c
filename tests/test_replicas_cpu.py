"""bench.py's replica plumbing (one process per GPU, no collective on the data path) with world_size 2
over gloo on the CPU: barrier, max-over-ranks timing and the summed fit count."""
import os
import sys

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def _worker(rank, world, port, q):
    os.environ.update(RANK=str(rank), WORLD_SIZE=str(world), LOCAL_RANK=str(rank),
                      MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port))
    sys.path.insert(0, ROOT)
    import bench
    r, w, local = bench.dist_init(None)
    bench.barrier(w)
    q.put((r, bench.allmax(1.0 + r, w), bench.allsum(16, w)))
    import torch.distributed as dist
    dist.destroy_process_group()


def test_two_replicas_over_gloo():
    import multiprocessing as mp
    import socket
    s = socket.socket()
    s.bind(("127.0.0.1", 0))
    port = s.getsockname()[1]
    s.close()
    ctx = mp.get_context("spawn")
    q = ctx.Queue()
    ps = [ctx.Process(target=_worker, args=(r, 2, port, q)) for r in range(2)]
    for p in ps:
        p.start()
    for p in ps:
        p.join(120)
        assert p.exitcode == 0
    out = sorted(q.get(timeout=5) for _ in range(2))
    assert [o[1] for o in out] == [2.0, 2.0]   # slowest rank's time
    assert [o[2] for o in out] == [32.0, 32.0]  # fits summed over replicas
