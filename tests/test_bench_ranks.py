"""Host logic of bench.py's N > 1 path on CPU: two gloo ranks (no GPU).

Each rank of a multi-GPU run answers against its own database replica; the
whole job's time is the maximum over ranks, and only rank 0 prints.  The
reference arm runs on rank 0 alone.
"""
import os
import socket

import pytest

torch = pytest.importorskip("torch")
import torch.distributed as dist  # noqa: E402
import torch.multiprocessing as mp  # noqa: E402


def _free_port() -> int:
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def _rank(rank, world, port, q):
    os.environ["MASTER_ADDR"] = "127.0.0.1"
    os.environ["MASTER_PORT"] = str(port)
    dist.init_process_group("gloo", rank=rank, world_size=world)
    try:
        import bench
        # rank r reports (1 + r, 5 - r): the maxima are (world, 5)
        q.put((rank, bench.max_over_ranks([1.0 + rank, 5.0 - rank], world)))
    finally:
        dist.destroy_process_group()


def test_max_over_two_gloo_ranks():
    ctx = mp.get_context("spawn")
    q = ctx.Queue()
    port = _free_port()
    procs = [ctx.Process(target=_rank, args=(r, 2, port, q)) for r in range(2)]
    for p in procs:
        p.start()
    try:
        got = sorted(q.get(timeout=120) for _ in procs)
    finally:
        for p in procs:
            p.join(timeout=60)
            if p.is_alive():
                p.kill()
    assert got == [(0, [2.0, 5.0]), (1, [2.0, 5.0])]
    assert all(p.exitcode == 0 for p in procs)


def test_max_over_one_rank_is_identity():
    import bench
    assert bench.max_over_ranks([3, 1.5], 1) == [3.0, 1.5]


def test_reference_arm_prints_on_rank0_only(capsys):
    import argparse

    import bench
    args = argparse.Namespace(gpus=2, steps=1, warmup=0)
    bench.run_reference(args, rank=1, world=2)
    assert capsys.readouterr().out == ""


def _rank_that_may_fail(rank, world, port, q):
    os.environ["MASTER_ADDR"] = "127.0.0.1"
    os.environ["MASTER_PORT"] = str(port)
    os.environ["RANK"] = str(rank)
    os.environ["WORLD_SIZE"] = str(world)
    import time

    import bench
    bench.init_ranks(timeout_s=5)
    if rank == 1:
        os._exit(3)                       # the replica dies before the exchange
    t0 = time.time()
    try:
        bench.max_over_ranks([1.0], world)
        q.put((rank, "no error", time.time() - t0))
    except Exception as e:  # noqa: BLE001 - the failure is what is checked
        q.put((rank, type(e).__name__, time.time() - t0))


def test_failed_rank_is_detected_by_the_others():
    """A rank that exits before the max-over-ranks exchange: the surviving
    rank's collective raises within the process group's timeout instead of
    hanging (host-side failure; no GPU involved)."""
    ctx = mp.get_context("spawn")
    q = ctx.Queue()
    port = _free_port()
    procs = [ctx.Process(target=_rank_that_may_fail, args=(r, 2, port, q)) for r in range(2)]
    for p in procs:
        p.start()
    try:
        rank, what, secs = q.get(timeout=180)
    finally:
        for p in procs:
            p.join(timeout=60)
            if p.is_alive():
                p.kill()
    assert rank == 0 and what != "no error" and secs < 60
    assert procs[1].exitcode == 3
