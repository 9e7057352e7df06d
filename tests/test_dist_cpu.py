"""The replica (N > 1) path of bench.py on CPU: two gloo ranks agree on the max-over-ranks time and
the summed launch count, and pass the barriers that bracket the timed region."""
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


def _rank(rank, world, port, out):
    os.environ.update(MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port), RANK=str(rank), WORLD_SIZE=str(world),
                      LOCAL_RANK=str(rank))
    sys.path.insert(0, ROOT)
    import bench

    ws, r, local = bench.dist_env()
    d = bench.Dist(ws, r, local, "gloo")
    d.barrier()
    mx = d.max(10.0 * (r + 1))
    sm = d.sum(r + 1)
    d.barrier()
    d.close()
    out.put((r, ws, mx, sm))


def test_two_gloo_ranks():
    torch = pytest.importorskip("torch")
    import torch.multiprocessing as mp

    ctx = mp.get_context("spawn")
    q = ctx.Queue()
    port = _free_port()
    procs = [ctx.Process(target=_rank, args=(r, 2, port, q)) for r in range(2)]
    for p in procs:
        p.start()
    for p in procs:
        p.join(timeout=120)
        assert p.exitcode == 0
    res = sorted(q.get(timeout=10) for _ in procs)
    assert [r for r, *_ in res] == [0, 1]
    for r, ws, mx, sm in res:
        assert ws == 2 and mx == 20.0 and sm == 3.0
