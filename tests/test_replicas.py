"""Multi-GPU replicas: routing by scene and the measurement reductions, run
as world-size-2 gloo process groups on the CPU (no GPU involved)."""
import os
import socket

import pytest

from mprgp_gb300 import replicas as R
from mprgp_gb300.workloads import Request


def _free_port():
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def test_split_window_keeps_scenes_together():
    reqs = [Request(0.1 * i, None, s, followup=(i > 3)) for i, s in
            enumerate([0, 1, 2, 3, 1, 2, 0, 3, 2, 5, 4, 5])]
    world = 3
    parts = [R.split_window(reqs, r, world) for r in range(world)]
    # every request exactly once, in arrival order within a rank
    assert sorted(id(q) for p in parts for q in p) == sorted(id(q) for q in reqs)
    for r, p in enumerate(parts):
        assert [q.t_arrive for q in p] == sorted(q.t_arrive for q in p)
        assert all(R.route_scene(q.scene, world) == r for q in p)
    # a scene's timesteps are all on one rank
    owner = {}
    for r, p in enumerate(parts):
        for q in p:
            assert owner.setdefault(q.scene, r) == r


def _worker(rank, world, port, out):
    import torch.distributed as dist
    os.environ.update(MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port), RANK=str(rank),
                      WORLD_SIZE=str(world), LOCAL_RANK=str(rank))
    dist.init_process_group("gloo", rank=rank, world_size=world)
    try:
        w, r, lr = R.rank_env()
        assert (w, r, lr) == (world, rank, rank)
        # rank 0 served 100 requests in 2 s, rank 1 served 100 in 4 s
        secs = 2.0 if rank == 0 else 4.0
        thr = R.aggregate_throughput(100.0, secs)
        mx = R.max_over_ranks(secs)
        sm = R.sum_over_ranks(1.0)
        out.put((rank, thr, mx, sm))
    finally:
        dist.destroy_process_group()


def test_gloo_world2_aggregation():
    mp = pytest.importorskip("torch.multiprocessing")
    ctx = mp.get_context("spawn")
    q = ctx.Queue()
    port = _free_port()
    procs = [ctx.Process(target=_worker, args=(r, 2, port, q)) for r in range(2)]
    for p in procs:
        p.start()
    for p in procs:
        p.join(timeout=120)
        assert p.exitcode == 0
    res = sorted(q.get(timeout=10) for _ in range(2))
    for rank, thr, mx, sm in res:
        assert thr == pytest.approx(200.0 / 4.0)   # all units over the slowest rank
        assert mx == 4.0 and sm == 2.0


def test_single_process_reductions_are_identity():
    assert R.aggregate_throughput(10.0, 2.0) == 5.0
