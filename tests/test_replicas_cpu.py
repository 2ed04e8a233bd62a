"""The multi-rank (replicas) logic of bench.py on CPU: world size 2 over gloo.

The k-eigenvalue path does not shard (one solve per GPU); `bench.py --gpus N` runs N
independent replicas and reduces over ranks only the timing (max) and the served rate
(sum).  These tests run that reduction with two gloo ranks, and the reference arm under
torchrun with two ranks: rank 0 alone times the CPU path and prints one JSON line.
"""
import json
import os
import socket
import subprocess
import sys

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def _free_port() -> int:
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def _rank_main(rank, world, port, out):
    import torch.distributed as dist
    sys.path.insert(0, ROOT)
    import bench
    dist.init_process_group("gloo", init_method=f"tcp://127.0.0.1:{port}", rank=rank, world_size=world)
    try:
        out.put((rank, bench.reduce_over_ranks(rank + 1.0, dist, "cpu", "max"),
                 bench.reduce_over_ranks(rank + 1.0, dist, "cpu", "sum")))
    finally:
        dist.destroy_process_group()


def test_reduce_over_ranks_gloo():
    import torch.multiprocessing as mp
    ctx = mp.get_context("spawn")
    out = ctx.Queue()
    port = _free_port()
    procs = [ctx.Process(target=_rank_main, args=(r, 2, port, out)) for r in range(2)]
    for p in procs:
        p.start()
    got = sorted(out.get(timeout=120) for _ in procs)
    for p in procs:
        p.join(timeout=60)
        assert p.exitcode == 0
    assert got == [(0, 2.0, 3.0), (1, 2.0, 3.0)]


def test_single_rank_reduction_is_identity():
    sys.path.insert(0, ROOT)
    import bench
    assert bench.reduce_over_ranks(1.5, None, "cpu", "max") == 1.5


@pytest.mark.timeout(600)
def test_reference_arm_two_ranks():
    from oracle import sn_cpu
    sn_cpu.build()
    cmd = [sys.executable, "-m", "torch.distributed.run", "--nnodes", "1", "--nproc-per-node", "2",
           "--master-addr", "127.0.0.1", "--master-port", str(_free_port()), os.path.join(ROOT, "bench.py"),
           "--impl", "reference", "--gpus", "2", "--steps", "1", "--warmup", "3", "--size", "16x16x8"]
    env = dict(os.environ, OMP_NUM_THREADS="2")
    res = subprocess.run(cmd, cwd=ROOT, capture_output=True, text=True, timeout=600, env=env)
    assert res.returncode == 0, res.stderr[-2000:]
    lines = [ln for ln in res.stdout.splitlines() if ln.startswith("{")]
    assert len(lines) == 1, res.stdout
    line = json.loads(lines[0])
    assert line["impl"] == "reference" and line["n_gpus"] == 2 and line["value"] > 0
    assert line["cpu_baseline"]["kind"] == "port"
