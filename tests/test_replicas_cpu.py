"""The multi-rank path of the benchmark on CPU: two gloo ranks (127.0.0.1),
each a replica with its own step time and work; the reduction gives the
maximum time and the summed work on every rank."""
import multiprocessing as mp
import os
import socket
import sys

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def _free_port() -> int:
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def _rank(rank, size, port, q):
    os.environ.update(RANK=str(rank), WORLD_SIZE=str(size), LOCAL_RANK=str(rank),
                      MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port))
    sys.path.insert(0, os.path.join(ROOT, "tests"))
    import conftest  # noqa: F401  (registers the package)
    from polgraw_gb300 import replicas
    assert replicas.init("gloo")
    replicas.barrier()
    t, u = replicas.reduce_step(1.0 + rank, 100.0 * (rank + 1))
    q.put((rank, t, u, replicas.world()))
    replicas.shutdown()


def test_two_gloo_ranks_reduce_time_and_work():
    pytest.importorskip("torch")
    port = _free_port()
    ctx = mp.get_context("spawn")
    q = ctx.Queue()
    procs = [ctx.Process(target=_rank, args=(r, 2, port, q)) for r in range(2)]
    for p in procs:
        p.start()
    for p in procs:
        p.join(120)
        assert p.exitcode == 0
    res = sorted(q.get(timeout=10) for _ in range(2))
    for rank, t, u, w in res:
        assert t == 2.0 and u == 300.0
        assert w == (rank, 2, rank)


def test_single_process_is_local():
    sys.path.insert(0, os.path.join(ROOT, "tests"))
    from polgraw_gb300 import replicas
    assert replicas.reduce_step(3.5, 7.0) == (3.5, 7.0)
