"""The bench's multi-rank path on the CPU: two `gloo` ranks (spawned processes) run the same
rendezvous, barrier and max/sum reductions the bench uses under torchrun, and split work the way
its replicas-only modes do (each rank its own seed; likelihood points rank::world)."""
import os
import socket
import sys
from pathlib import Path

import pytest

ROOT = Path(__file__).resolve().parents[1]


def _free_port() -> int:
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def _worker(rank, world, port, q):
    os.environ.update(MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port), RANK=str(rank),
                      WORLD_SIZE=str(world), LOCAL_RANK=str(rank))
    sys.path.insert(0, str(ROOT))
    import numpy as np

    import bench

    w, r, local, dist = bench.dist_setup()
    mx = bench.reduce_max(dist, 10.0 * (r + 1))
    sm = bench.reduce_sum(dist, float(r + 1))
    bench.barrier(dist)
    pts = np.arange(64)[r::w]
    q.put((r, w, local, mx, sm, pts.tolist()))
    dist.destroy_process_group()


def test_two_gloo_ranks_reduce_and_split():
    torch = pytest.importorskip("torch")
    mp = torch.multiprocessing.get_context("spawn")
    q = mp.Queue()
    port = _free_port()
    procs = [mp.Process(target=_worker, args=(r, 2, port, q)) for r in range(2)]
    for p in procs:
        p.start()
    out = sorted(q.get(timeout=120) for _ in procs)
    for p in procs:
        p.join(timeout=60)
        assert p.exitcode == 0
    assert [o[0] for o in out] == [0, 1] and all(o[1] == 2 for o in out)
    assert all(o[3] == 20.0 for o in out)          # max over ranks (the bench's timing rule)
    assert all(o[4] == 3.0 for o in out)           # whole-job sum of the ranks' work
    assert sorted(out[0][5] + out[1][5]) == list(range(64))
    assert not set(out[0][5]) & set(out[1][5])


def test_single_rank_needs_no_process_group():
    sys.path.insert(0, str(ROOT))
    import bench

    env = {k: os.environ.pop(k) for k in ("WORLD_SIZE", "RANK", "LOCAL_RANK") if k in os.environ}
    try:
        w, r, local, dist = bench.dist_setup()
        assert (w, r, local, dist) == (1, 0, 0, None)
        assert bench.reduce_max(dist, 2.5) == 2.5 and bench.reduce_sum(dist, 4.0) == 4.0
        bench.barrier(dist)
    finally:
        os.environ.update(env)
