"""bench.py's multi-rank plumbing on CPU (gloo, world size 2): every rank aligns its own
seeded shard (weak scaling, no collective on the data path); step times are combined with a
max and pair counts with a sum."""
import os
import socket

import pytest


def _free_port() -> int:
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def _worker(rank: int, world: int, port: int, q):
    os.environ.update(MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port), RANK=str(rank), WORLD_SIZE=str(world),
                      LOCAL_RANK=str(rank))
    import sys
    from pathlib import Path
    sys.path.insert(0, str(Path(__file__).resolve().parent.parent))
    import bench
    d = bench.Dist(world, backend="gloo")
    d.barrier()
    mx = d.max(float(10 * (rank + 1)))
    sm = d.sum(float(rank + 1))
    b = bench.make_batch(2, 8, rank)
    d.close()
    q.put((rank, mx, sm, bytes(b.seq[:64])))


def test_two_ranks_combine_times_and_counts():
    pytest.importorskip("torch")
    import multiprocessing as mp
    ctx = mp.get_context("spawn")
    q = ctx.Queue()
    port = _free_port()
    procs = [ctx.Process(target=_worker, args=(r, 2, port, q)) for r in range(2)]
    for p in procs:
        p.start()
    out = [q.get(timeout=120) for _ in procs]
    for p in procs:
        p.join(timeout=60)
        assert p.exitcode == 0
    out.sort()
    assert all(o[1] == 20.0 for o in out)   # max over ranks
    assert all(o[2] == 3.0 for o in out)    # sum over ranks
    assert out[0][3] != out[1][3]           # each rank aligns its own seeded shard
