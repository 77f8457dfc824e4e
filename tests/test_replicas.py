"""N>1 replicas (bench.py): each rank renders its own frames, no data-path
collective; the job's value is the segments of all ranks over the slowest
rank's time.  Run as two gloo ranks on the CPU."""
import os
import socket
import sys
from pathlib import Path

import pytest
import torch.multiprocessing as mp

ROOT = Path(__file__).resolve().parents[1]


def _free_port() -> int:
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def _rank(rank: int, world: int, port: int, out):
    os.environ.update(MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port), RANK=str(rank), WORLD_SIZE=str(world),
                      LOCAL_RANK=str(rank))
    sys.path.insert(0, str(ROOT))
    import bench

    dist = bench.Dist(world, "gloo")
    # rank r took (r + 1) * 10 ms for (r + 1) * 1e6 segments
    value, ms, segs = bench.aggregate(dist, (rank + 1) * 10.0, (rank + 1) * 1e6)
    dist.barrier()
    dist.close()
    out.put((rank, value, ms, segs))


def test_two_replicas_aggregate_with_gloo():
    ctx = mp.get_context("spawn")
    q = ctx.Queue()
    port = _free_port()
    procs = [ctx.Process(target=_rank, args=(r, 2, port, q)) for r in range(2)]
    for p in procs:
        p.start()
    results = [q.get(timeout=120) for _ in procs]
    for p in procs:
        p.join(timeout=60)
        assert p.exitcode == 0
    for rank, value, ms, segs in results:
        assert ms == pytest.approx(20.0)       # slowest rank
        assert segs == pytest.approx(3e6)      # all ranks' work
        assert value == pytest.approx(3e6 / 20e-3 / 1e9)


def test_single_rank_aggregate_is_local():
    sys.path.insert(0, str(ROOT))
    import bench

    value, ms, segs = bench.aggregate(bench.Dist(1, "gloo"), 4.0, 2e6)
    assert (ms, segs) == (4.0, 2e6) and value == pytest.approx(0.5)
