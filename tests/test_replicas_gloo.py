"""The multi-GPU path is replicas only (independent systems, no collective in
the step).  Its host logic -- rank set-up, the barrier, the slowest rank's
time and the whole-job throughput -- runs here as two gloo processes on CPU."""
import os
import socket
import sys

import pytest
import torch.multiprocessing as mp

from conftest import ROOT


def _free_port():
    s = socket.socket()
    s.bind(("127.0.0.1", 0))
    p = s.getsockname()[1]
    s.close()
    return p


def _rank(rank, ws, port, q):
    os.environ.update({"RANK": str(rank), "WORLD_SIZE": str(ws), "LOCAL_RANK": str(rank),
                       "MASTER_ADDR": "127.0.0.1", "MASTER_PORT": str(port)})
    sys.path.insert(0, ROOT)
    import bench
    dist, r, w = bench.dist_init("gloo")
    bench.barrier(dist)
    # rank r took (r + 1) ms per step on its own replica of 1000 beads
    value, ms = bench.replica_result(dist, w, 1000, float(r + 1))
    q.put((r, w, value, ms))
    dist.destroy_process_group()


def test_replica_throughput_uses_slowest_rank():
    ws, port = 2, _free_port()
    ctx = mp.get_context("spawn")
    q = ctx.Queue()
    procs = [ctx.Process(target=_rank, args=(r, ws, port, q)) for r in range(ws)]
    for p in procs:
        p.start()
    out = [q.get(timeout=120) for _ in range(ws)]
    for p in procs:
        p.join(timeout=60)
        assert p.exitcode == 0
    for r, w, value, ms in out:
        assert w == 2
        assert ms == pytest.approx(2.0)  # the slowest rank
        assert value == pytest.approx(2 * 1000 / 2e-3)
