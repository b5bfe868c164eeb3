"""The N > 1 path of bench.py on CPU: two gloo ranks (127.0.0.1) reduce their timed-region seconds to
the maximum, as the GPU ranks do over NCCL; the reference arm does its work on rank 0 only."""
import os
import socket
import sys

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def _free_port() -> int:
    with socket.socket() as sk:
        sk.bind(("127.0.0.1", 0))
        return sk.getsockname()[1]


def _rank_main(rank, world, port, q):
    import torch
    import torch.distributed as dist

    sys.path.insert(0, ROOT)
    import bench

    os.environ.update(MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port))
    dist.init_process_group("gloo", rank=rank, world_size=world)
    t = bench.max_over_ranks(torch, 1.0 + 2.0 * rank, dist, "cpu")
    q.put((rank, t))
    dist.destroy_process_group()


def test_max_over_ranks_gloo_world2():
    import torch.multiprocessing as mp

    ctx = mp.get_context("spawn")
    q = ctx.Queue()
    port = _free_port()
    procs = [ctx.Process(target=_rank_main, args=(r, 2, port, q)) for r in range(2)]
    for p in procs:
        p.start()
    got = dict(q.get(timeout=120) for _ in procs)
    for p in procs:
        p.join(timeout=60)
        assert p.exitcode == 0
    assert got == {0: 3.0, 1: 3.0}


def test_max_over_ranks_single_process():
    import torch

    sys.path.insert(0, ROOT)
    import bench

    assert bench.max_over_ranks(torch, 2.5, None, "cpu") == 2.5


def test_reference_arm_other_ranks_exit_without_work(monkeypatch):
    sys.path.insert(0, ROOT)
    import bench

    monkeypatch.setenv("RANK", "1")

    class Args:
        case = "mixed24"
        steps = 1
        warmup = 0
        gpus = 2

    assert bench.run_reference(Args()) == 0


def test_serving_requests_target_resident_objects():
    """The request stream of the serving leg: Poisson arrivals, ~30% assemblies, and every step targets
    one of the four most recently submitted objects (so that it stays resident under the HBM cap)."""
    import numpy as np

    sys.path.insert(0, ROOT)
    import bench

    reqs = bench.serving_requests(7, 400, 30.0)
    t = np.array([r["t"] for r in reqs])
    assert np.all(np.diff(t) > 0)
    assert abs(len(reqs) / t[-1] - 30.0) < 6.0
    n_asm = sum(r["type"] == "assembly" for r in reqs)
    assert 0.2 < n_asm / len(reqs) < 0.4
    submitted = []
    for k, r in enumerate(reqs):
        if r["type"] == "assembly":
            submitted.append(k)
        else:
            assert r["target"] in submitted[-4:]
            assert len(r["p"]) == 3 * reqs[r["target"]]["mesh"].nV
