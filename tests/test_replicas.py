"""Multi-GPU host logic (replicas only): member sharding and the whole-job
rate, on CPU ranks over gloo (world size 2).  No GPU is involved; the data
path has no collective, so these are the only cross-rank operations."""
import os
import socket

import pytest

from wrf_gb300.replicas import job_rate, reduce_max, reduce_sum, shard_members


def test_shard_members_covers_and_balances():
    sizes = [5, 9, 1, 7, 3, 3, 8, 2, 6, 4]
    for world in (1, 2, 3, 4, 8):
        parts = shard_members(sizes, world)
        assert len(parts) == world
        flat = sorted(q for p in parts for q in p)
        assert flat == list(range(len(sizes)))
        loads = [sum(sizes[q] for q in p) for p in parts]
        # LPT greedy: max load within the largest item of the mean
        assert max(loads) - min(loads) <= max(sizes)
    assert shard_members(sizes, 2) == shard_members(list(sizes), 2)  # deterministic


def test_shard_members_uneven_ensemble():
    from wrf_gb300 import cases
    specs = cases.ensemble_members(seed=4)
    cells = [s[0] * s[1] * (s[2] - 1) for s in specs]
    parts = shard_members(cells, 4)
    loads = [sum(cells[q] for q in p) for p in parts]
    assert max(loads) / min(loads) < 1.05


def _free_port():
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def _worker(rank, world, port, out):
    import torch.distributed as dist
    os.environ["MASTER_ADDR"] = "127.0.0.1"
    os.environ["MASTER_PORT"] = str(port)
    dist.init_process_group("gloo", rank=rank, world_size=world)
    try:
        rate, total, slowest = job_rate(dist, local_units=100.0 * (rank + 1), local_seconds=2.0 + rank)
        out[rank] = (rate, total, slowest, reduce_max(dist, rank), reduce_sum(dist, 1.0))
    finally:
        dist.destroy_process_group()


def test_job_rate_gloo_two_ranks():
    mp = pytest.importorskip("torch.multiprocessing")
    ctx = mp.get_context("spawn")
    mgr = ctx.Manager()
    out = mgr.dict()
    port = _free_port()
    procs = [ctx.Process(target=_worker, args=(r, 2, port, out)) for r in range(2)]
    for p in procs:
        p.start()
    for p in procs:
        p.join(timeout=120)
        assert p.exitcode == 0
    for r in range(2):
        rate, total, slowest, mx, n = out[r]
        assert total == 300.0 and slowest == 3.0 and rate == 100.0
        assert mx == 1.0 and n == 2.0


def test_job_rate_single_process():
    assert job_rate(None, 50.0, 2.0) == (25.0, 50.0, 2.0)


def test_bench_reference_arm_two_ranks():
    """`bench.py --impl reference` under torchrun with 2 CPU ranks (gloo):
    rank 0 alone times the CPU path and prints one JSON line."""
    import json
    import subprocess
    import sys
    root = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
    env = dict(os.environ, CUDA_VISIBLE_DEVICES="")
    cmd = [sys.executable, "-m", "torch.distributed.run", "--nnodes=1", "--nproc-per-node", "2",
           "--master-addr", "127.0.0.1", "--master-port", str(_free_port()),
           os.path.join(root, "bench.py"), "--impl", "reference", "--workload", "c1",
           "--steps", "1", "--warmup", "0", "--ref-steps", "1", "--gpus", "2"]
    r = subprocess.run(cmd, capture_output=True, text=True, timeout=600, env=env, cwd=root)
    assert r.returncode == 0, r.stderr[-2000:]
    lines = [ln for ln in r.stdout.splitlines() if ln.startswith("{")]
    assert len(lines) == 1
    d = json.loads(lines[0])
    assert d["impl"] == "reference" and d["value"] > 0 and d["cpu_baseline"]["kind"] == "port"
    assert d["e2e"]["h2d_bytes_per_step"] == 0 and d["e2e"]["d2h_bytes_per_step"] == 0
