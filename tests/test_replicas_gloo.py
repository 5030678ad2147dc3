"""The multi-GPU path is replicas only (one independent simulation per rank, no
data-path collective). What the ranks share is the timing: a barrier around the timed
region and the max over ranks, from which rank 0 reports the whole-job rate. Checked
here with two gloo ranks on CPU."""
import os
import socket
import sys
from pathlib import Path

import pytest

ROOT = Path(__file__).resolve().parent.parent


def _free_port():
    s = socket.socket()
    s.bind(("127.0.0.1", 0))
    p = s.getsockname()[1]
    s.close()
    return p


def _worker(rank, world, port, out):
    os.environ.update({"RANK": str(rank), "WORLD_SIZE": str(world), "LOCAL_RANK": str(rank),
                       "MASTER_ADDR": "127.0.0.1", "MASTER_PORT": str(port)})
    sys.path.insert(0, str(ROOT))
    import bench
    w, r, local, dist = bench.dist_setup(None, backend="gloo")
    bench.barrier(dist)
    ms_local = 100.0 + 50.0 * r            # rank 1 is the slow one
    rate, ms = bench.replica_rate(dist, w, 10, ms_local)
    bench.barrier(dist)
    out.put((r, w, rate, ms))
    dist.destroy_process_group()


def test_two_gloo_replicas_report_the_slowest_rank():
    torch = pytest.importorskip("torch")
    mp = torch.multiprocessing.get_context("spawn")
    q = mp.Queue()
    port = _free_port()
    procs = [mp.Process(target=_worker, args=(r, 2, port, q)) for r in range(2)]
    for p in procs:
        p.start()
    res = sorted(q.get(timeout=120) for _ in procs)
    for p in procs:
        p.join(timeout=60)
        assert p.exitcode == 0
    for r, w, rate, ms in res:
        assert w == 2
        assert ms == 150.0                    # max over ranks
        assert rate == pytest.approx(2 * 10 / 0.150)
