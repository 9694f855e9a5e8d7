"""The multi-GPU path of bench.py on the host, without a GPU: the visibility
pass does not shard, so N GPUs run N replicas of the frame, and the only
host logic is the reduction of the ranks' times (the slowest replica sets
the step) and the reference arm's rule that rank 0 alone works.  Two
``gloo`` ranks in spawned processes stand in for two GPUs."""
from __future__ import annotations

import io
import multiprocessing as mp
import socket
import sys
from contextlib import redirect_stdout
from pathlib import Path
from types import SimpleNamespace

ROOT = Path(__file__).resolve().parents[1]


def _free_port() -> int:
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def _rank(rank: int, world: int, port: int, values, out) -> None:
    import os
    os.environ.update(MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port))
    sys.path.insert(0, str(ROOT))
    import torch.distributed as dist
    import bench
    dist.init_process_group("gloo", rank=rank, world_size=world)
    try:
        out.put((rank, [bench.max_over_ranks(v, dist, "cpu") for v in values[rank]]))
    finally:
        dist.destroy_process_group()


def test_max_over_ranks_with_two_gloo_ranks():
    """Every rank gets the slowest rank's time, value by value (the device
    step time, then the two end-to-end times, in the same order on all ranks)."""
    ctx = mp.get_context("spawn")
    out = ctx.Queue()
    values = [[0.137, 0.210, 0.188], [0.141, 0.176, 0.201]]
    port = _free_port()
    procs = [ctx.Process(target=_rank, args=(r, 2, port, values, out)) for r in range(2)]
    for p in procs:
        p.start()
    got = dict(out.get(timeout=120) for _ in procs)
    for p in procs:
        p.join(timeout=60)
        assert p.exitcode == 0
    expect = [max(a, b) for a, b in zip(*values)]
    assert got[0] == got[1] == expect


def test_max_over_ranks_without_a_process_group():
    sys.path.insert(0, str(ROOT))
    import bench
    assert bench.max_over_ranks(0.25, None, "cpu") == 0.25


def test_reference_arm_runs_on_rank_zero_only():
    """Under torchrun the reference arm's other ranks exit without work or output."""
    sys.path.insert(0, str(ROOT))
    import bench
    buf = io.StringIO()
    with redirect_stdout(buf):
        bench.run_reference(SimpleNamespace(gpus=2, steps=1, warmup=3), rank=1)
    assert buf.getvalue() == ""
