"""Replica aggregation of bench.py on two gloo ranks (CPU, no GPU): the
timed region takes the max over ranks and the work the sum, as the bench
reports for N replicas."""
import multiprocessing as mp
import os
import socket
import sys
from pathlib import Path

ROOT = Path(__file__).resolve().parent.parent


def _free_port():
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def _rank_main(rank, ws, port, q):
    os.environ.update({"RANK": str(rank), "WORLD_SIZE": str(ws), "LOCAL_RANK": str(rank),
                       "MASTER_ADDR": "127.0.0.1", "MASTER_PORT": str(port)})
    sys.path.insert(0, str(ROOT))
    import bench
    r = bench.Ranks(ws)
    r.barrier()
    out = (r.max(1.5 + rank), r.sum(10.0 * (rank + 1)), bench.dist_env())
    r.close()
    q.put((rank, out))


def test_two_gloo_ranks_max_and_sum():
    ctx = mp.get_context("spawn")
    q = ctx.Queue()
    port = _free_port()
    procs = [ctx.Process(target=_rank_main, args=(r, 2, port, q)) for r in range(2)]
    for p in procs:
        p.start()
    got = dict(q.get(timeout=120) for _ in procs)
    for p in procs:
        p.join(timeout=60)
        assert p.exitcode == 0
    for rank in (0, 1):
        mx, sm, env = got[rank]
        assert mx == 2.5 and sm == 30.0
        assert env == (2, rank, rank)


def test_single_process_is_a_no_op():
    sys.path.insert(0, str(ROOT))
    import bench
    r = bench.Ranks(1)
    r.barrier()
    assert r.max(3.0) == 3.0 and r.sum(4.0) == 4.0
    r.close()
