"""The multi-rank path of bench.py on CPU: two gloo ranks (world size 2),
rendezvous on 127.0.0.1.  The path runs independent replicas (no data-path
collective): the only cross-rank operations are the barrier around the
timed region and the max-over-ranks time / sum-over-ranks cells of the
whole-job value; the reference arm runs on rank 0 only."""
from __future__ import annotations

import importlib.util
import os
import socket
import sys
from pathlib import Path

import pytest

torch = pytest.importorskip("torch")
ROOT = Path(__file__).resolve().parents[1]


def _free_port():
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def _bench():
    spec = importlib.util.spec_from_file_location("bench_under_test", ROOT / "bench.py")
    mod = importlib.util.module_from_spec(spec)
    spec.loader.exec_module(mod)
    return mod


def _worker(rank, world, port, q):
    os.environ.update(RANK=str(rank), WORLD_SIZE=str(world), LOCAL_RANK=str(rank), MASTER_ADDR="127.0.0.1",
                      MASTER_PORT=str(port))
    b = _bench()
    r, w, local = b.dist_env()
    dist = b.init_dist(w)
    b.barrier(dist)
    # rank-specific timings and cells: the job value uses the slowest rank
    value, ms = b.aggregate(dist, cells_local=1000.0 * (r + 1), ms_local=10.0 + r)
    mx = b.allmax(dist, float(r))
    sm = b.allsum(dist, float(r + 1))

    class A:
        n, steps, warmup = 8, 1, 0
    # the reference arm: rank 1 returns at once (would otherwise import the oracle and print)
    ref = b.run_reference(A) if r == 1 else None
    b.barrier(dist)
    dist.destroy_process_group()
    q.put((r, w, value, ms, mx, sm, ref))


def test_two_gloo_ranks():
    ctx = torch.multiprocessing.get_context("spawn")
    q = ctx.Queue()
    port = _free_port()
    procs = [ctx.Process(target=_worker, args=(r, 2, port, q)) for r in range(2)]
    for p in procs:
        p.start()
    out = sorted(q.get(timeout=120) for _ in procs)
    for p in procs:
        p.join(timeout=60)
        assert p.exitcode == 0
    for r, w, value, ms, mx, sm, ref in out:
        assert w == 2
        assert ms == 11.0                          # max over ranks
        assert value == pytest.approx(3000.0 / 0.011)  # all cells over the slowest time
        assert mx == 1.0 and sm == 3.0
        assert ref is None


def test_single_rank_needs_no_process_group():
    b = _bench()
    assert b.init_dist(1) is None
    value, ms = b.aggregate(None, 500.0, 5.0)
    assert ms == 5.0 and value == pytest.approx(1e5)
