"""bench.py's multi-rank logic on CPU with the gloo backend, world size 2:
each rank owns a disjoint block of walkers, the step time is the maximum over
ranks and the job's pair count is the sum over ranks."""
import os
import socket
import sys

import pytest

torch = pytest.importorskip("torch")
import torch.distributed as dist  # noqa: E402
import torch.multiprocessing as mp  # noqa: E402

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def _free_port():
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def _worker(rank, world, port, q):
    sys.path.insert(0, ROOT)
    import bench
    os.environ.update(MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port))
    dist.init_process_group("gloo", rank=rank, world_size=world)
    try:
        w = bench.rank_walkers(rank, 16)
        t = bench.reduce_over_ranks(0.5 + rank, "max")
        n = bench.reduce_over_ranks(1000 * (rank + 1), "sum")
        q.put((rank, w, t, n))
    finally:
        dist.destroy_process_group()


def test_two_ranks_gloo():
    ctx = mp.get_context("spawn")
    q = ctx.Queue()
    port = _free_port()
    procs = [ctx.Process(target=_worker, args=(r, 2, port, q)) for r in range(2)]
    for p in procs:
        p.start()
    got = sorted(q.get(timeout=120) for _ in procs)
    for p in procs:
        p.join(timeout=60)
        assert p.exitcode == 0
    (r0, w0, t0, n0), (r1, w1, t1, n1) = got
    assert (r0, r1) == (0, 1)
    assert w0 == list(range(16)) and w1 == list(range(16, 32))
    assert t0 == t1 == 1.5
    assert n0 == n1 == 3000


def test_single_process_identity():
    sys.path.insert(0, ROOT)
    import bench
    assert bench.reduce_over_ranks(2.5, "max") == 2.5
    assert bench.rank_walkers(0, 3) == [0, 1, 2]
