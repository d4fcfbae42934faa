"""The multi-GPU arrangement of the benchmark: independent replicas, one per
rank, whose only exchange is the maximum of the timed region over the ranks
(gloo), and a reference arm that runs on rank 0 alone.  Tested here with two
CPU ranks over gloo; no GPU is involved."""
import os
import socket
import subprocess
import sys

import pytest
import torch.multiprocessing as tmp

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def _free_port():
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def _rank_main(rank, ws, port, out):
    os.environ.update(MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port), WORLD_SIZE=str(ws), RANK=str(rank),
                      LOCAL_RANK=str(rank))
    sys.path.insert(0, ROOT)
    import torch.distributed as dist
    import bench
    dist.init_process_group("gloo")
    ms = 10.0 * (rank + 1)          # the ranks' own timed regions
    m = bench.replica_max(ms)
    rate = bench.job_rate(ws, 1000, 5, m)
    out.put((rank, m, rate))
    dist.barrier()
    dist.destroy_process_group()


def test_replica_timing_is_the_maximum_over_two_ranks():
    ws, port = 2, _free_port()
    ctx = tmp.get_context("spawn")
    q = ctx.Queue()
    procs = [ctx.Process(target=_rank_main, args=(r, ws, port, q)) for r in range(ws)]
    for p in procs:
        p.start()
    res = sorted(q.get(timeout=120) for _ in range(ws))
    for p in procs:
        p.join(timeout=60)
        assert p.exitcode == 0
    # both ranks see the slowest rank's time; the rate counts every rank's box
    assert [m for _, m, _ in res] == [20.0, 20.0]
    assert all(abs(r - 2 * 1000 * 5 / 0.020) < 1e-6 for _, _, r in res)


def test_single_rank_needs_no_process_group():
    sys.path.insert(0, ROOT)
    import bench
    env = {k: v for k, v in os.environ.items() if k not in ("WORLD_SIZE", "RANK", "LOCAL_RANK")}
    old = dict(os.environ)
    try:
        os.environ.clear()
        os.environ.update(env)
        assert bench.replica_max(12.5) == 12.5
    finally:
        os.environ.clear()
        os.environ.update(old)


@pytest.mark.parametrize("rank", [1])
def test_reference_arm_runs_on_rank_zero_only(rank):
    """Under torchrun the reference arm's other ranks exit 0 without work or output."""
    env = dict(os.environ, WORLD_SIZE="2", RANK=str(rank), LOCAL_RANK=str(rank))
    r = subprocess.run([sys.executable, os.path.join(ROOT, "bench.py"), "--impl", "reference", "--gpus", "2"],
                       env=env, capture_output=True, text=True, timeout=300)
    assert r.returncode == 0, r.stderr
    assert r.stdout.strip() == ""
