"""The multi-process path of bench.py on host-only ranks (gloo, world size 2).

A single DM-QR does not shard, so `bench.py --gpus N` runs N independent
replicas: a barrier on both sides of the timed region, the time taken as the
maximum over ranks, one JSON line from rank 0.  The reference arm runs on
rank 0 alone and the other ranks exit without work.  These tests drive that
host logic with the gloo backend; the GPU replicas themselves run only on a
GPU machine.
"""
import importlib.util
import json
import os
import socket
import subprocess
import sys

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def _free_port():
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def _load_bench():
    spec = importlib.util.spec_from_file_location("bench_module", os.path.join(ROOT, "bench.py"))
    mod = importlib.util.module_from_spec(spec)
    spec.loader.exec_module(mod)
    return mod


def _max_worker(rank, world, port, out):
    os.environ.update(MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port), RANK=str(rank),
                      WORLD_SIZE=str(world), LOCAL_RANK=str(rank))
    sys.path.insert(0, ROOT)
    bench = _load_bench()
    r, w, _ = bench.dist_setup(world)
    bench.barrier(w)
    out[r] = bench.max_over_ranks(1.5 + r, w)  # rank 1 holds the larger time
    bench.barrier(w)
    import torch.distributed as dist

    dist.destroy_process_group()


def test_max_over_ranks_gloo():
    import torch
    import torch.multiprocessing as mp

    if torch.cuda.is_available():
        pytest.skip("host-only ranks: this test covers the gloo fallback")
    ctx = mp.get_context("spawn")
    manager = ctx.Manager()
    out = manager.dict()
    port = _free_port()
    procs = [ctx.Process(target=_max_worker, args=(r, 2, port, out)) for r in range(2)]
    for p in procs:
        p.start()
    for p in procs:
        p.join(timeout=120)
        assert p.exitcode == 0
    assert dict(out) == {0: 2.5, 1: 2.5}


def test_reference_arm_two_ranks():
    """torchrun with two ranks: rank 0 prints the one JSON line of the
    reference arm, rank 1 exits 0 without work."""
    import torch

    if torch.cuda.is_available():
        pytest.skip("host-only ranks: this test covers the gloo fallback")
    port = _free_port()
    cmd = [sys.executable, "-m", "torch.distributed.run", "--nnodes=1", "--nproc-per-node", "2",
           "--master-addr", "127.0.0.1", "--master-port", str(port),
           os.path.join(ROOT, "bench.py"), "--impl", "reference", "--gpus", "2", "--steps", "1",
           "--warmup", "0", "--workload", "graded1k"]
    env = dict(os.environ, OMP_NUM_THREADS="1")
    r = subprocess.run(cmd, capture_output=True, text=True, timeout=600, cwd=ROOT, env=env)
    assert r.returncode == 0, r.stderr[-2000:]
    lines = [ln for ln in r.stdout.splitlines() if ln.startswith("{")]
    assert len(lines) == 1, r.stdout
    d = json.loads(lines[0])
    assert d["impl"] == "reference" and d["n_gpus"] == 2
    assert d["value"] > 0 and d["cpu_baseline"]["kind"] == "port"
    assert d["e2e"]["h2d_bytes_per_step"] == 0
