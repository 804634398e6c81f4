"""Multi-rank logic of bench.py on CPU (gloo, world size 2).

Each rank processes its own frame (weak scaling); the only collectives are the
timing barrier and the element-wise maximum of the per-rank step times.
"""

import io
import json
import os
import socket
import sys
from contextlib import redirect_stdout
from pathlib import Path

import pytest

torch = pytest.importorskip("torch")
import torch.distributed as dist  # noqa: E402
import torch.multiprocessing as tmp  # noqa: E402

ROOT = Path(__file__).resolve().parent.parent


def _free_port():
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def _worker(rank, world, port, q):
    sys.path.insert(0, str(ROOT))
    os.environ.update(MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port))
    dist.init_process_group("gloo", rank=rank, world_size=world)
    try:
        import bench

        # rank r reports timings that differ per rank; every rank must see the maximum
        got = bench.max_over_ranks([1.0 + rank, 10.0 - rank, 0.5 * rank], dist)
        # the reference arm: only rank 0 prints, the other ranks return without work
        buf = io.StringIO()

        class A:
            gpus, steps, warmup = world, 0, 0

        if rank != 0:
            with redirect_stdout(buf):
                bench.run_reference(A, rank, world)
        q.put((rank, got, buf.getvalue()))
        dist.barrier()
    finally:
        dist.destroy_process_group()


def test_max_over_ranks_and_reference_arm_gloo_world2():
    world = 2
    ctx = tmp.get_context("spawn")
    q = ctx.Queue()
    port = _free_port()
    procs = [ctx.Process(target=_worker, args=(r, world, port, q)) for r in range(world)]
    for p in procs:
        p.start()
    res = {}
    for _ in range(world):
        rank, got, out = q.get(timeout=120)
        res[rank] = (got, out)
    for p in procs:
        p.join(timeout=60)
        assert p.exitcode == 0
    for rank in range(world):
        assert res[rank][0] == [2.0, 10.0, 0.5]
    assert res[1][1] == ""


def test_max_over_ranks_single_process():
    sys.path.insert(0, str(ROOT))
    import bench

    assert bench.max_over_ranks([3.0, 4.0], None) == [3.0, 4.0]


def test_block_plan_is_per_rank_frame():
    sys.path.insert(0, str(ROOT))
    import bench

    plan = bench.block_plan(2048, 2048, 1024, (5, 11))
    assert len(plan) == 4
    # every output pixel of the rank's frame is written exactly once
    cover = {}
    for (_ir, _ic, _tr, _tc, orr, occ) in plan:
        cover[(orr, occ)] = cover.get((orr, occ), 0) + 1
    assert sum((r[1] - r[0]) * (c[1] - c[0]) for (r, c) in cover) == 2048 * 2048
    json.dumps(plan)
