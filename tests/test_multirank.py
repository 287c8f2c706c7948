"""The bench's multi-process path on CPU: two gloo ranks, each owning its own
trajectories (disjoint ids), no data-path collective; the whole-job rate is
every rank's units over the slowest rank's timed interval."""
import os
import socket
import sys

import pytest
import torch.multiprocessing as mp

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def _free_port():
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def _rank(rank, world, port, q):
    import torch.distributed as dist
    sys.path.insert(0, ROOT)
    os.environ.update(MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port))
    dist.init_process_group("gloo", rank=rank, world_size=world)
    import bench
    elapsed = [2.0, 3.0][rank]  # the second rank is slower
    e = bench.max_over_ranks(elapsed)
    rate = bench.whole_job_rate(512, 2, world, e)
    # trajectory ids owned by each rank do not overlap (rank * B offset)
    B = 4
    ids = list(range(rank * B, rank * B + B))
    q.put((rank, e, rate, ids))
    dist.barrier()
    dist.destroy_process_group()


def test_two_gloo_ranks_aggregate_max_time_and_whole_job_rate():
    pytest.importorskip("torch.distributed")
    ctx = mp.get_context("spawn")
    q = ctx.Queue()
    port = _free_port()
    procs = [ctx.Process(target=_rank, args=(r, 2, port, q)) for r in range(2)]
    for p in procs:
        p.start()
    out = sorted(q.get(timeout=120) for _ in procs)
    for p in procs:
        p.join(timeout=60)
        assert p.exitcode == 0
    for rank, e, rate, ids in out:
        assert e == 3.0
        assert rate == pytest.approx(2 * 512 * 2 / 3.0)
    assert set(out[0][3]).isdisjoint(out[1][3])


def test_single_process_rate_needs_no_process_group():
    sys.path.insert(0, ROOT)
    import bench
    assert bench.max_over_ranks(1.5) == 1.5
    assert bench.whole_job_rate(512, 2, 1, 4.0) == 256.0
