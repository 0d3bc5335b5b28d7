"""The multi-GPU bench path's host logic on two CPU ranks (gloo): every rank assembles its own
strand, the job's value is the units of all ranks over the slowest rank's time."""

from __future__ import annotations

import importlib.util
import socket
from pathlib import Path

import pytest

torch = pytest.importorskip("torch")
ROOT = Path(__file__).resolve().parents[1]


def _bench():
    spec = importlib.util.spec_from_file_location("_xk_bench", ROOT / "bench.py")
    mod = importlib.util.module_from_spec(spec)
    spec.loader.exec_module(mod)
    return mod


def _free_port() -> int:
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def _rank(rank: int, world: int, port: int, q):
    import torch.distributed as dist

    dist.init_process_group("gloo", init_method=f"tcp://127.0.0.1:{port}", rank=rank, world_size=world)
    try:
        bench = _bench()
        # rank r: times (1 + r, 10 - r), units 100 + r
        t, n = bench.rank_aggregate([1.0 + rank, 10.0 - rank], [100.0 + rank])
        q.put((rank, t, n))
    finally:
        dist.destroy_process_group()


def test_rank_aggregate_two_gloo_ranks():
    ctx = torch.multiprocessing.get_context("spawn")
    q = ctx.Queue()
    port = _free_port()
    procs = [ctx.Process(target=_rank, args=(r, 2, port, q)) for r in range(2)]
    for p in procs:
        p.start()
    out = [q.get(timeout=120) for _ in procs]
    for p in procs:
        p.join(timeout=60)
        assert p.exitcode == 0
    for rank, t, n in out:
        assert t == [2.0, 10.0]  # the slowest rank's time, each entry
        assert n == [201.0]      # the units of both ranks


def test_rank_aggregate_single_process_is_identity():
    t, n = _bench().rank_aggregate([1.5, 2.5], [7])
    assert t == [1.5, 2.5] and n == [7.0]


def test_reference_arm_runs_on_every_core():
    """``bench.py --impl reference`` times the NumPy port in one spawned process per host core, each
    on its own slab of every wire (CPU; a small strand keeps it to seconds)."""
    import json
    import os
    import subprocess
    import sys

    env = dict(os.environ, XK_REF_BUDGET_S="60")
    out = subprocess.run([sys.executable, str(ROOT / "bench.py"), "--impl", "reference", "--workload", "strand37",
                          "--steps", "1", "--warmup", "1"], capture_output=True, text=True, timeout=600, env=env,
                         cwd=ROOT)
    assert out.returncode == 0, out.stderr[-2000:]
    line = json.loads(out.stdout.strip().splitlines()[-1])
    cores = len(os.sched_getaffinity(0)) if hasattr(os, "sched_getaffinity") else os.cpu_count()
    assert line["impl"] == "reference" and line["value"] > 0
    assert line["cpu_baseline"]["cores"] == line["config"]["processes"] == min(cores, 128 // 2)
    assert line["e2e"]["value"] == line["value"]
