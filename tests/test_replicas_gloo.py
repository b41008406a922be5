"""The multi-GPU path of bench.py is replicas only: each rank advances its own
suspension and the process group carries just the barrier and the
max-over-ranks of the timed region.  Checked here with two gloo ranks on the
CPU (no GPU): every rank sees the slowest rank's time and the same whole-job
value."""
import os
import socket
import sys

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def _free_port():
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def _rank(rank, world, port, out):
    os.environ.update(MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port), WORLD_SIZE=str(world), RANK=str(rank),
                      LOCAL_RANK=str(rank))
    sys.path.insert(0, ROOT)
    import bench
    w, r, local, dist, torch = bench.dist_setup(backend="gloo")
    assert (w, r) == (world, rank)
    mine = 1.0 + 0.5 * rank                      # seconds this rank "took"
    dist.barrier()
    slowest = bench.max_over_ranks(mine, dist, torch, "cpu")
    out.put((rank, slowest, bench.replica_value(4096, 10, w, slowest)))
    dist.destroy_process_group()


def test_two_gloo_ranks_agree_on_the_slowest_time():
    torch = pytest.importorskip("torch")
    import torch.multiprocessing as mp
    ctx = mp.get_context("spawn")
    q = ctx.Queue()
    port = _free_port()
    procs = [ctx.Process(target=_rank, args=(r, 2, port, q)) for r in range(2)]
    for p in procs:
        p.start()
    res = sorted(q.get(timeout=120) for _ in procs)
    for p in procs:
        p.join(timeout=60)
        assert p.exitcode == 0
    assert [r[1] for r in res] == [1.5, 1.5]
    assert all(abs(r[2] - 4096 * 10 * 2 / 1.5) < 1e-6 for r in res)
