"""The N > 1 path of bench.py: one independent replica per rank, a gloo
barrier and the max of the per-rank times (world_size 2 on the CPU)."""
import os
import socket
import sys

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def _free_port():
    s = socket.socket()
    s.bind(("127.0.0.1", 0))
    port = s.getsockname()[1]
    s.close()
    return port


def _rank(rank, world, port, q):
    os.environ.update(MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port), RANK=str(rank), WORLD_SIZE=str(world),
                      LOCAL_RANK=str(rank))
    sys.path.insert(0, ROOT)
    import bench
    r, w, local = bench.dist_env()
    d = bench.Dist(w)
    d.barrier()
    m = d.max(float(10 + rank))
    d.close()
    q.put((r, w, local, m))


def test_two_rank_barrier_and_max():
    torch = pytest.importorskip("torch")
    mp = torch.multiprocessing.get_context("spawn")
    q = mp.Queue()
    port = _free_port()
    procs = [mp.Process(target=_rank, args=(r, 2, port, q)) for r in range(2)]
    for p in procs:
        p.start()
    for p in procs:
        p.join(120)
    res = sorted(q.get(timeout=10) for _ in range(2))
    assert [x[0] for x in res] == [0, 1]
    assert all(x[1] == 2 for x in res)
    assert all(x[3] == 11.0 for x in res)  # every rank sees the max over ranks
    assert all(p.exitcode == 0 for p in procs)
