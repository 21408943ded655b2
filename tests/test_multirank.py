"""The N > 1 host path of bench.py on CPU: two ranks over gloo (127.0.0.1) take the barrier and
the max over ranks that bracket the timed region, and the reference arm runs on rank 0 only.
Replicas only: no rank exchanges simulation data."""
import multiprocessing as mp
import os
import socket
import sys
from pathlib import Path

import pytest

ROOT = Path(__file__).resolve().parent.parent


def _free_port():
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def _rank(rank, world, port, q):
    os.environ.update(RANK=str(rank), WORLD_SIZE=str(world), LOCAL_RANK=str(rank),
                      MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port))
    sys.path.insert(0, str(ROOT))
    import bench
    r, w, local = bench.dist_env()
    d = bench.Dist(w, local, "gloo")
    d.barrier()
    m = d.max(1.5 + r)          # each rank's timed seconds; the job's is the slowest
    d.barrier()
    d.close()
    q.put((r, w, m))


def test_two_ranks_barrier_and_max_over_gloo():
    pytest.importorskip("torch.distributed")
    ctx = mp.get_context("spawn")
    q = ctx.Queue()
    port = _free_port()
    procs = [ctx.Process(target=_rank, args=(r, 2, port, q)) for r in range(2)]
    for p in procs:
        p.start()
    out = sorted(q.get(timeout=120) for _ in procs)
    for p in procs:
        p.join(timeout=60)
        assert p.exitcode == 0
    assert out == [(0, 2, 2.5), (1, 2, 2.5)]


def test_reference_arm_runs_on_rank_zero_only(capsys):
    sys.path.insert(0, str(ROOT))
    import bench

    class Args:
        workload, steps, warmup = "two_body_large", 1, 0
    bench.run_reference(Args(), rank=1, world=2, local=1)   # rank 1: no work, no output
    assert capsys.readouterr().out == ""
