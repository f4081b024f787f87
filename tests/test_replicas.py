"""The multi-rank path of bench.py (replicas: one grid per rank, no data-path
collective) on CPU: two gloo ranks agree on the slowest rank's time and on the
whole-job throughput."""
import os
import socket
import sys

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def _free_port() -> int:
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def _rank(rank, world, port, q):
    sys.path.insert(0, ROOT)
    os.environ.update(MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port), RANK=str(rank), WORLD_SIZE=str(world),
                      LOCAL_RANK=str(rank))
    import torch.distributed as dist
    import bench
    r, w, local = bench.dist_env()
    dist.init_process_group("gloo", rank=r, world_size=w)
    t = bench.max_over_ranks(1.5 + rank, w, device="cpu")
    v = bench.replicas_value(1000.0, w, t)
    dist.barrier()
    dist.destroy_process_group()
    q.put((r, w, local, t, v))


def test_two_gloo_ranks_take_the_slowest_time():
    import multiprocessing as mp
    ctx = mp.get_context("spawn")
    q = ctx.Queue()
    port = _free_port()
    ps = [ctx.Process(target=_rank, args=(k, 2, port, q)) for k in range(2)]
    for p in ps:
        p.start()
    out = sorted(q.get(timeout=120) for _ in ps)
    for p in ps:
        p.join(timeout=60)
        assert p.exitcode == 0
    assert [o[0] for o in out] == [0, 1] and all(o[1] == 2 for o in out)
    assert all(o[3] == pytest.approx(2.5) for o in out)          # max over ranks
    assert all(o[4] == pytest.approx(2 * 1000.0 / 2.5) for o in out)


def test_single_rank_needs_no_process_group():
    sys.path.insert(0, ROOT)
    import bench
    assert bench.max_over_ranks(3.0, 1) == 3.0
    assert bench.replicas_value(10.0, 1, 2.0) == 5.0
