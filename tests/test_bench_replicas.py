"""The replica path of bench.py at world size 2 on the CPU (gloo ranks): each
rank reads its rank from the launcher's environment and the timed region's
result is the maximum over the ranks, the path's only collective.  The
trajectories do not exchange data, so nothing else crosses ranks."""
import os
import socket
import sys

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def _free_port():
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def _rank(rank, world, port, queue):
    os.environ.update(RANK=str(rank), WORLD_SIZE=str(world), LOCAL_RANK=str(rank), MASTER_ADDR="127.0.0.1",
                      MASTER_PORT=str(port))
    sys.path.insert(0, ROOT)
    import torch.distributed as dist
    import bench
    dist.init_process_group("gloo", rank=rank, world_size=world)
    r, w, local = bench.dist_info()
    ms = bench.barrier_max(10.0 + 5.0 * rank, w)  # rank 1 is the slower one
    queue.put((r, w, local, ms))
    dist.destroy_process_group()


def test_timing_is_the_max_over_two_gloo_ranks():
    mp = pytest.importorskip("torch.multiprocessing")
    ctx = mp.get_context("spawn")
    queue = ctx.Queue()
    port = _free_port()
    procs = [ctx.Process(target=_rank, args=(r, 2, port, queue)) for r in range(2)]
    for p in procs:
        p.start()
    got = sorted(queue.get(timeout=180) for _ in procs)
    for p in procs:
        p.join(timeout=60)
    assert [p.exitcode for p in procs] == [0, 0]
    assert got == [(0, 2, 0, 15.0), (1, 2, 1, 15.0)]


def test_single_process_needs_no_collective():
    sys.path.insert(0, ROOT)
    import bench
    assert bench.barrier_max(3.5, 1) == 3.5
