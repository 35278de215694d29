"""The N>1 path of bench.py: independent replicas, one rank per GPU, with no
data-path collective.  The host side (rendezvous, barrier, max over ranks of
the step time, the whole-job aggregate, rank 0 alone printing the reference
arm) runs here as two gloo ranks on CPU; no kernel is launched."""
import io
import os
import socket
import sys
import types
from contextlib import redirect_stdout

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def _free_port():
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def _rank_main(rank, world, port, q):
    sys.path.insert(0, ROOT)
    os.environ.update(RANK=str(rank), WORLD_SIZE=str(world), LOCAL_RANK=str(rank), MASTER_ADDR="127.0.0.1",
                      MASTER_PORT=str(port))
    import bench
    r, w, local = bench.dist_env()
    dist = bench.init_dist(w)
    try:
        bench.barrier(dist)
        # rank-local step times; the job is as slow as its slowest replica
        ms = bench.max_over_ranks(dist, 10.0 + 5.0 * r)
        value = bench.job_gbs(w, 4, ms)
        buf = io.StringIO()
        args = types.SimpleNamespace(gpus=w, steps=1, warmup=0)
        if r != 0:
            with redirect_stdout(buf):
                bench.run_reference(args, r, w)
        bench.barrier(dist)
        q.put((r, local, ms, value, buf.getvalue()))
    finally:
        dist.destroy_process_group()


def test_two_gloo_replicas():
    mp = pytest.importorskip("torch.multiprocessing")
    ctx = mp.get_context("spawn")
    q = ctx.Queue()
    port = _free_port()
    world = 2
    procs = [ctx.Process(target=_rank_main, args=(r, world, port, q)) for r in range(world)]
    for p in procs:
        p.start()
    out = [q.get(timeout=120) for _ in range(world)]
    for p in procs:
        p.join(timeout=60)
        assert p.exitcode == 0
    import bench
    for r, local, ms, value, printed in out:
        assert local == r
        assert ms == 15.0  # max over ranks, seen identically by every rank
        assert value == pytest.approx(world * bench.STEP_BYTES * 4 / 15e-3 / 1e9)
        assert printed == ""  # only rank 0 runs and prints the reference arm


def test_single_rank_needs_no_process_group(monkeypatch):
    for k in ("RANK", "WORLD_SIZE", "LOCAL_RANK"):
        monkeypatch.delenv(k, raising=False)
    import bench
    assert bench.dist_env() == (0, 1, 0)
    assert bench.init_dist(1) is None
    assert bench.max_over_ranks(None, 3.5) == 3.5
    assert bench.job_gbs(1, 2, 1000.0) == pytest.approx(2 * bench.STEP_BYTES / 1e9)
