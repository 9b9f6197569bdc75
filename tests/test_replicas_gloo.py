"""The multi-GPU path of bench.py runs independent replicas; its only
cross-rank step is the MAX reduction of the timed regions.  Checked here
with two gloo ranks on the CPU."""
import os
import socket
import sys

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def free_port():
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def _rank(rank, world, port, out):
    import torch.distributed as dist
    sys.path.insert(0, ROOT)
    import bench
    os.environ.update(MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port))
    dist.init_process_group("gloo", rank=rank, world_size=world)
    # rank r timed 100 steps in (1000 + 500 r) ms and 10 e2e calls in (2 + r) s
    value, e2e, total = bench.aggregate(1000.0 + 500.0 * rank, 2.0 + rank, 100, 10, world, dist, "cpu")
    out.put((rank, value, e2e, total))
    dist.barrier()
    dist.destroy_process_group()


def test_max_over_ranks_two_gloo_ranks():
    torch = pytest.importorskip("torch")
    mp = torch.multiprocessing.get_context("spawn")
    q = mp.Queue()
    port = free_port()
    procs = [mp.Process(target=_rank, args=(r, 2, port, q)) for r in range(2)]
    for p in procs:
        p.start()
    res = sorted(q.get(timeout=120) for _ in procs)
    for p in procs:
        p.join(timeout=60)
        assert p.exitcode == 0
    for rank, value, e2e, total in res:
        assert total == 1500.0                      # the slowest rank's region
        assert value == pytest.approx(2 * 100 / 1.5)  # all ranks' steps / max time
        assert e2e == pytest.approx(2 * 10 / 3.0)


def test_single_rank_needs_no_process_group():
    sys.path.insert(0, ROOT)
    import bench
    value, e2e, total = bench.aggregate(500.0, 1.0, 50, 5, 1, None, "cpu")
    assert (value, e2e, total) == (100.0, 5.0, 500.0)
