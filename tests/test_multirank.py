"""The multi-rank host path of bench.py on CPU: two gloo ranks.

With N GPUs bench.py runs N independent replicas (the instances shard with
no data-path collective): the ranks only meet in a barrier and in the max
(time) and sum (units processed) over ranks, and for the reference arm rank
0 alone prints.  Both are exercised here with world_size 2 on 127.0.0.1.
"""
import json
import os
import socket
import subprocess
import sys

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def free_port():
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def _rank(rank, port, out):
    os.environ.update({"MASTER_ADDR": "127.0.0.1", "MASTER_PORT": str(port), "RANK": str(rank),
                       "WORLD_SIZE": "2", "LOCAL_RANK": str(rank)})
    sys.path.insert(0, ROOT)
    import bench
    world, r, local = bench.dist_setup()
    bench.barrier(world)
    res = (r, bench.allmax(float(r + 1), world), bench.allsum(float(r + 1), world))
    bench.barrier(world)
    out.put(res)
    import torch.distributed as dist
    dist.destroy_process_group()


def test_max_and_sum_over_two_gloo_ranks():
    mp = pytest.importorskip("torch.multiprocessing")
    ctx = mp.get_context("spawn")
    q = ctx.Queue()
    port = free_port()
    procs = [ctx.Process(target=_rank, args=(r, port, q)) for r in range(2)]
    for p in procs:
        p.start()
    res = sorted(q.get(timeout=120) for _ in procs)
    for p in procs:
        p.join(timeout=60)
        assert p.exitcode == 0
    assert res == [(0, 2.0, 3.0), (1, 2.0, 3.0)]


def test_reference_arm_prints_once_under_torchrun():
    port = free_port()
    r = subprocess.run([sys.executable, "-m", "torch.distributed.run", "--nnodes=1", "--nproc-per-node", "2",
                        "--master-addr", "127.0.0.1", "--master-port", str(port), "bench.py",
                        "--impl", "reference", "--workload", "tiny", "--gpus", "2", "--steps", "1",
                        "--warmup", "1"], cwd=ROOT, capture_output=True, text=True, timeout=300)
    assert r.returncode == 0, r.stderr[-2000:]
    lines = [l for l in r.stdout.splitlines() if l.startswith("{")]
    assert len(lines) == 1
    d = json.loads(lines[0])
    assert d["impl"] == "reference" and d["n_gpus"] == 2 and d["value"] > 0
    assert d["cpu_baseline"]["kind"] in ("port", "reference")
