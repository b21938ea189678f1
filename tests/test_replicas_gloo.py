"""The multi-GPU path is replicas only (every rank steps its own copy of the workload; no data-path
collective): its host logic, run as world-size-2 gloo process groups on the CPU."""
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


def _worker(rank, world, port, out):
    import torch.distributed as dist

    sys.path.insert(0, ROOT)
    import bench

    dist.init_process_group("gloo", init_method=f"tcp://127.0.0.1:{port}", rank=rank, world_size=world)
    try:
        res = bench.max_over_ranks([1.0 + rank, 10.0 * rank, 5.0 - rank])
        out.put((rank, res))
    finally:
        dist.destroy_process_group()


def test_max_over_ranks_world2():
    import torch.multiprocessing as mp

    ctx = mp.get_context("spawn")
    q = ctx.Queue()
    port = _free_port()
    procs = [ctx.Process(target=_worker, args=(r, 2, port, q)) for r in range(2)]
    for p in procs:
        p.start()
    got = dict(q.get(timeout=120) for _ in procs)
    for p in procs:
        p.join(timeout=60)
        assert p.exitcode == 0
    assert got[0] == got[1] == [2.0, 10.0, 5.0]


def test_max_over_ranks_without_group():
    sys.path.insert(0, ROOT)
    import bench

    assert bench.max_over_ranks([3.0, 1.0]) == [3.0, 1.0]


def test_reference_arm_under_torchrun_world2():
    """bench.py --impl reference under torchrun with two ranks: rank 0 alone runs the CPU reference arm and
    prints one JSON line; rank 1 exits 0 without work."""
    port = _free_port()
    env = dict(os.environ)
    env.pop("CUDA_VISIBLE_DEVICES", None)
    cmd = [sys.executable, "-m", "torch.distributed.run", "--nnodes=1", "--nproc-per-node", "2", "--master-addr",
           "127.0.0.1", "--master-port", str(port), os.path.join(ROOT, "bench.py"), "--impl", "reference",
           "--workload", "cube10", "--gpus", "2", "--steps", "1", "--warmup", "0", "--cpu-seconds", "1"]
    r = subprocess.run(cmd, capture_output=True, text=True, timeout=600, cwd=ROOT, env=env)
    assert r.returncode == 0, r.stderr[-2000:]
    lines = [l for l in r.stdout.splitlines() if l.startswith("{")]
    assert len(lines) == 1, r.stdout
    d = json.loads(lines[0])
    assert d["impl"] == "reference" and d["n_gpus"] == 2 and d["value"] > 0
    assert d["e2e"]["h2d_bytes_per_step"] == 0 and d["cpu_baseline"]["kind"] == "port"
