"""The multi-rank path of the benchmark on CPU: two gloo ranks (127.0.0.1),
each with its own block of the sky, step time and work; the reduction gives
the maximum time and the summed work on every rank; the blocks are
contiguous, disjoint and cover the sky."""
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
    from polgraw_gb300 import shards
    assert shards.init("gloo")
    shards.barrier()
    t, u = shards.reduce_step(1.0 + rank, 100.0 * (rank + 1))
    sky = [(1, mm, nn) for mm in range(-3, 4) for nn in range(-3, 4)]
    q.put((rank, t, u, shards.world(), shards.shard(sky, rank, size)))
    shards.shutdown()


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
    for rank, t, u, w, blk in res:
        assert t == 2.0 and u == 300.0
        assert w == (rank, 2, rank)
    sky = [(1, mm, nn) for mm in range(-3, 4) for nn in range(-3, 4)]
    assert res[0][4] + res[1][4] == sky          # contiguous, disjoint, covering


def test_single_process_is_local():
    sys.path.insert(0, os.path.join(ROOT, "tests"))
    from polgraw_gb300 import shards
    assert shards.reduce_step(3.5, 7.0) == (3.5, 7.0)


def test_shard_blocks():
    sys.path.insert(0, os.path.join(ROOT, "tests"))
    from polgraw_gb300 import shards
    t = list(range(10))
    assert [shards.shard(t, r, 3) for r in range(3)] == [[0, 1, 2], [3, 4, 5], [6, 7, 8, 9]]
    assert [shards.shard(t, r, 2, 4) for r in range(2)] == [[0, 1, 2, 3], [4, 5, 6, 7]]
    assert shards.shard(t, 0, 1, 4) == [0, 1, 2, 3] and shards.shard(t, 0, 1) == t
