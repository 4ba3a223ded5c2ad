"""The multi-process (N > 1) host logic of bench.py on CPU: two gloo ranks, as
torchrun launches them, reduce their timings with max_over_ranks (the slowest
replica sets the whole-job time) and read their rank from the environment."""
import os
import socket
import sys

import pytest

torch = pytest.importorskip("torch")
import torch.multiprocessing as mp  # noqa: E402

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def _free_port():
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def _rank_main(rank, world, port, q):
    os.environ.update({"RANK": str(rank), "WORLD_SIZE": str(world), "LOCAL_RANK": str(rank),
                       "MASTER_ADDR": "127.0.0.1", "MASTER_PORT": str(port)})
    sys.path.insert(0, ROOT)
    import torch.distributed as dist

    import bench

    dist.init_process_group("gloo", rank=rank, world_size=world)
    try:
        r, w, local = bench.dist_env()
        vals = bench.max_over_ranks([float(r), 10.0 - r, 3.5])
        dist.barrier()
        q.put((rank, r, w, local, vals))
    finally:
        dist.destroy_process_group()


def test_two_gloo_ranks_take_the_max():
    ctx = mp.get_context("spawn")
    q = ctx.Queue()
    port = _free_port()
    procs = [ctx.Process(target=_rank_main, args=(r, 2, port, q)) for r in range(2)]
    for p in procs:
        p.start()
    got = sorted(q.get(timeout=120) for _ in procs)
    for p in procs:
        p.join(timeout=60)
        assert p.exitcode == 0
    for rank, r, w, local, vals in got:
        assert (r, w, local) == (rank, 2, rank)
        assert vals == [1.0, 10.0, 3.5]


def test_one_rank_is_unchanged():
    sys.path.insert(0, ROOT)
    import bench

    assert bench.max_over_ranks([2.0, 5.0]) == [2.0, 5.0]
