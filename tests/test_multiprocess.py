"""The multi-rank path of bench.py on CPU (gloo, world size 2): every rank
runs an independent replica, the job time is the slowest rank's and the rate
counts the work of all ranks; under torchrun only rank 0 runs and prints the
reference arm."""
import json
import os
import socket
import subprocess
import sys

import pytest

torch = pytest.importorskip("torch")
ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def _free_port():
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def _worker(rank, ws, port, out):
    import torch.distributed as dist
    sys.path.insert(0, ROOT)
    import bench
    os.environ.update(MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port))
    dist.init_process_group("gloo", rank=rank, world_size=ws)
    ms = 10.0 + 5.0 * rank  # rank 1 is the slow one
    job_ms = bench.max_over_ranks(ms, ws)
    out[rank] = (job_ms, bench.aggregate_rate(1000.0, ws, job_ms))
    dist.barrier()
    dist.destroy_process_group()


def test_replicas_take_the_slowest_rank_and_count_all_work():
    import torch.multiprocessing as mp
    ws = 2
    mgr = mp.get_context("spawn").Manager()  # no fork of this (threaded) process
    out = mgr.dict()
    mp.spawn(_worker, args=(ws, _free_port(), out), nprocs=ws, join=True)
    for r in range(ws):
        job_ms, rate = out[r]
        assert job_ms == 15.0
        assert rate == pytest.approx(1000.0 * ws / 15e-3)


def test_reference_arm_runs_on_rank_zero_only():
    env = dict(os.environ, WORLD_SIZE="2", RANK="1", LOCAL_RANK="1")
    r = subprocess.run([sys.executable, os.path.join(ROOT, "bench.py"), "--impl", "reference", "--steps", "1",
                        "--warmup", "0"], capture_output=True, text=True, env=env, timeout=600)
    assert r.returncode == 0, r.stderr[-2000:]
    assert r.stdout.strip() == ""


def test_reference_arm_prints_its_line():
    r = subprocess.run([sys.executable, os.path.join(ROOT, "bench.py"), "--impl", "reference", "--steps", "1",
                        "--warmup", "0"], capture_output=True, text=True, timeout=900)
    assert r.returncode == 0, r.stderr[-2000:]
    line = json.loads(r.stdout.strip().splitlines()[-1])
    assert line["impl"] == "reference" and line["value"] > 0
    assert line["e2e"]["h2d_bytes_per_step"] == 0 and line["cpu_baseline"]["kind"] == "port"
