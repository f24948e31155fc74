"""The N > 1 path of bench.py: independent replicas, one per rank, joined only by a gloo
barrier and a max-over-ranks time with summed units (no data-path collective)."""
from __future__ import annotations

import multiprocessing as mp
import os
import socket

from conftest import REPO


def _free_port() -> int:
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def _worker(rank: int, ws: int, port: int, q) -> None:
    os.environ.update(RANK=str(rank), WORLD_SIZE=str(ws), LOCAL_RANK=str(rank),
                      MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port))
    import sys
    sys.path.insert(0, str(REPO))
    import bench
    d = bench.Dist("gloo")
    d.barrier()
    value, ms = bench.aggregate(d, units_local=100.0 * (rank + 1), ms_local=10.0 * (rank + 1))
    q.put((rank, value, ms))
    d.barrier()
    d.close()


def test_replica_aggregation_world_size_2():
    ctx = mp.get_context("spawn")
    q = ctx.Queue()
    port = _free_port()
    ps = [ctx.Process(target=_worker, args=(r, 2, port, q)) for r in range(2)]
    for p in ps:
        p.start()
    for p in ps:
        p.join(120)
        assert p.exitcode == 0
    got = sorted(q.get(timeout=10) for _ in range(2))
    # units summed over ranks (100 + 200), time = the slowest rank (20 ms)
    for rank, value, ms in got:
        assert ms == 20.0
        assert abs(value - 300.0 / 0.020) < 1e-6
