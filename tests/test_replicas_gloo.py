"""The multi-GPU path of bench.py is replicas only (independent bodies, no
data-path collective): each rank runs the same workload and the job's time is
the slowest rank's.  Here two gloo ranks on the CPU exercise that reduction
and the whole-job throughput formula."""
import os
import socket

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def _free_port():
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def _rank_main(rank, world, port, q):
    import sys
    sys.path.insert(0, ROOT)
    os.environ.update(MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port), RANK=str(rank), WORLD_SIZE=str(world),
                      LOCAL_RANK=str(rank))
    import torch.distributed as dist
    import bench
    dist.init_process_group("gloo", rank=rank, world_size=world)
    try:
        r, lr, w = bench.dist_info()
        slowest = bench.max_over_ranks(100.0 + 10.0 * rank)
        q.put((r, lr, w, slowest, bench.replica_throughput(1000, 5, w, slowest)))
    finally:
        dist.destroy_process_group()


def test_two_gloo_ranks_take_the_slowest_time():
    import torch.multiprocessing as mp
    ctx = mp.get_context("spawn")
    q = ctx.Queue()
    port = _free_port()
    procs = [ctx.Process(target=_rank_main, args=(r, 2, port, q)) for r in range(2)]
    for p in procs:
        p.start()
    for p in procs:
        p.join(timeout=120)
        assert p.exitcode == 0
    out = sorted(q.get(timeout=5) for _ in range(2))
    assert [o[0] for o in out] == [0, 1] and all(o[2] == 2 for o in out)
    for o in out:
        assert o[3] == pytest.approx(110.0)
        assert o[4] == pytest.approx(1000 * 5 * 2 / 0.110)


def test_single_process_needs_no_group():
    import sys
    sys.path.insert(0, ROOT)
    import bench
    assert bench.max_over_ranks(3.5) == 3.5
