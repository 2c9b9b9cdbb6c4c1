"""The multi-rank host logic of ``bench.py`` on CPU: two ``gloo`` ranks.

``bench.py --gpus N`` runs N independent replicas (one volume per rank, weak
scaling, no data-path collective). Each rank times its own calls; the line's
time is the maximum over ranks, and rank 0 alone prints. These tests run that
reduction (``bench.max_over_ranks``, the function the GPU arm calls under NCCL)
in two spawned processes over ``gloo``, and check the rank handling of the
reference arm and the per-rank inputs."""

import os
import socket
import sys
from types import SimpleNamespace

import numpy as np
import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def _free_port() -> int:
    with socket.socket(socket.AF_INET, socket.SOCK_STREAM) as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def _rank_main(rank: int, world: int, port: int, queue) -> None:
    os.environ["MASTER_ADDR"] = "127.0.0.1"
    os.environ["MASTER_PORT"] = str(port)
    sys.path.insert(0, ROOT)
    import torch.distributed as dist

    import bench

    dist.init_process_group("gloo", rank=rank, world_size=world)
    try:
        # per-rank durations: the slowest rank sets each figure
        out = bench.max_over_ranks([1.5 + rank, 20.0 - 5.0 * rank, 0.25], dist, "cpu")
        dist.barrier()
        queue.put((rank, out))
    finally:
        dist.destroy_process_group()


def test_max_over_ranks_two_gloo_ranks():
    import torch.multiprocessing as mp

    ctx = mp.get_context("spawn")
    queue = ctx.Queue()
    port = _free_port()
    procs = [ctx.Process(target=_rank_main, args=(r, 2, port, queue), daemon=True) for r in range(2)]
    for p in procs:
        p.start()
    try:
        got = dict(queue.get(timeout=180) for _ in procs)
    finally:
        for p in procs:
            p.join(timeout=60)
            if p.is_alive():  # a rank that never returned: end it (it is this test's own child)
                p.terminate()
                p.join(timeout=10)
    assert all(p.exitcode == 0 for p in procs)
    assert got[0] == got[1] == [2.5, 20.0, 0.25]


def test_max_over_ranks_single_rank_is_identity():
    sys.path.insert(0, ROOT)
    import bench

    assert bench.max_over_ranks([3.0, 1.0], None, "cpu") == [3.0, 1.0]


def test_reference_arm_runs_on_rank_zero_only():
    sys.path.insert(0, ROOT)
    import bench

    args = SimpleNamespace(workload="bm4d256", steps=1, warmup=0)
    assert bench.run_reference(args, rank=1, world=2) is None


def test_replicas_get_distinct_volumes():
    """Weak scaling: rank r denoises the phantom of seed r, so the ranks' work is
    independent and equal in size."""
    sys.path.insert(0, ROOT)
    import bench

    c0, n0 = bench.make_input("bm3d256", seed=0)
    c1, n1 = bench.make_input("bm3d256", seed=1)
    assert n0.shape == n1.shape and n0.dtype == n1.dtype == np.float32
    assert not np.array_equal(n0, n1)
