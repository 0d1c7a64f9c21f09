"""CPU tests of the multi-rank (replicas) path of bench.py with the gloo
backend, world size 2: process-group set-up from the torchrun environment,
the barrier around the timed region, the max over ranks of the measured time,
the whole-job value, and the reference arm's rank handling (rank 0 alone
times the CPU path; the other ranks exit at once)."""
import os
import socket
import subprocess
import sys

import pytest

from conftest import ROOT


def _free_port():
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def _worker(rank, world, port, q):
    os.environ.update(RANK=str(rank), WORLD_SIZE=str(world), LOCAL_RANK=str(rank), MASTER_ADDR="127.0.0.1",
                      MASTER_PORT=str(port))
    sys.path.insert(0, ROOT)
    import torch.distributed as dist
    import bench
    r, w, _ = bench.dist_setup()
    bench.barrier(w)
    t_ms = 1000.0 * (1.0 + r)  # rank r "took" 1 + r seconds
    m = bench.allmax(t_ms, w)
    q.put((r, w, m, bench.replica_value(5, 8, w, m)))
    bench.barrier(w)
    dist.destroy_process_group()


def test_two_replicas_over_gloo():
    import torch.multiprocessing as mp
    ctx = mp.get_context("spawn")
    q = ctx.Queue()
    port = _free_port()
    procs = [ctx.Process(target=_worker, args=(r, 2, port, q)) for r in range(2)]
    for p in procs:
        p.start()
    out = [q.get(timeout=120) for _ in procs]
    for p in procs:
        p.join(timeout=60)
        assert p.exitcode == 0
    out.sort()
    assert [o[0] for o in out] == [0, 1]
    for r, w, m, v in out:
        assert w == 2
        assert m == 2000.0  # the slowest rank's time
        assert v == pytest.approx(5 * 8 * 2 / 2.0)  # all ranks' pairs over the max time


def test_reference_arm_other_ranks_exit_without_work():
    env = dict(os.environ, RANK="1", WORLD_SIZE="2", LOCAL_RANK="1", MASTER_ADDR="127.0.0.1",
               MASTER_PORT=str(_free_port()))
    r = subprocess.run([sys.executable, os.path.join(ROOT, "bench.py"), "--impl", "reference", "--steps", "1",
                        "--warmup", "0"], env=env, capture_output=True, text=True, timeout=120)
    assert r.returncode == 0, r.stderr
    assert r.stdout.strip() == ""
