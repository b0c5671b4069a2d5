"""Multi-rank host logic of bench.py on CPU (gloo, world size 2).

Replicas only: each rank assembles its own copy of the workload, so the only cross-rank
steps are the barrier and the max-over-ranks of the timed region; the whole-job rate is all
ranks' elements over the slowest rank's time.
"""
import json
import os
import socket
import subprocess
import sys

import pytest
import torch.multiprocessing as mp

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def _free_port():
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def _worker(rank, world, port, q):
    import torch.distributed as dist
    sys.path.insert(0, ROOT)
    import bench
    os.environ.update(MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port))
    dist.init_process_group("gloo", rank=rank, world_size=world)
    try:
        t = 1.0 + rank  # rank 1 is the slow one
        slowest = bench.max_over_ranks(t)
        dist.barrier()
        q.put((rank, slowest, bench.whole_job_rate(world, 1_000_000, slowest)))
    finally:
        dist.destroy_process_group()


def test_max_over_ranks_and_whole_job_rate_gloo():
    port = _free_port()
    ctx = mp.get_context("spawn")
    q = ctx.Queue()
    procs = [ctx.Process(target=_worker, args=(r, 2, port, q)) for r in range(2)]
    for p in procs:
        p.start()
    res = sorted(q.get(timeout=120) for _ in procs)
    for p in procs:
        p.join(timeout=60)
        assert p.exitcode == 0
    assert [r[1] for r in res] == [2.0, 2.0]          # both ranks see the slowest time
    assert all(abs(r[2] - 1.0) < 1e-12 for r in res)  # 2 ranks x 1 M elements / 2 s = 1 Melem/s


def test_single_process_is_identity():
    sys.path.insert(0, ROOT)
    import bench
    assert bench.max_over_ranks(3.5) == 3.5
    assert bench.whole_job_rate(1, 2_000_000, 2.0) == 1.0


def test_reference_arm_under_torchrun_prints_one_line():
    """`bench.py --impl reference` launched with 2 ranks: rank 0 alone times the CPU port and
    prints one JSON line; the other rank exits 0 without work."""
    pytest.importorskip("torch.distributed.run")
    cmd = [sys.executable, "-m", "torch.distributed.run", "--nnodes=1", "--nproc-per-node", "2",
           "--master-addr", "127.0.0.1", "--master-port", str(_free_port()), "bench.py",
           "--impl", "reference", "--gpus", "2", "--steps", "1", "--warmup", "0", "--config", "c1"]
    env = dict(os.environ, OMP_NUM_THREADS="2")
    r = subprocess.run(cmd, cwd=ROOT, capture_output=True, text=True, timeout=600, env=env)
    assert r.returncode == 0, r.stderr[-2000:]
    lines = [l for l in r.stdout.splitlines() if l.startswith("{")]
    assert len(lines) == 1
    d = json.loads(lines[0])
    assert d["impl"] == "reference" and d["n_gpus"] == 2 and d["value"] > 0
    assert d["e2e"]["h2d_bytes_per_step"] == 0 and d["cpu_baseline"]["kind"] == "port"
    # the reference arm times the full workload mesh and never maps the product library
    assert d["config"]["same_config"] is True and "19,200 elements" in d["config"]["workload"]
    assert all(p.startswith("oracle/") for p in d["native_so_loaded"]), d["native_so_loaded"]
