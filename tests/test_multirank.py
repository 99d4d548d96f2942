"""The bench's multi-rank path on CPU: world_size 2 over gloo (127.0.0.1).  The path is
replicas only (the (xi, m) matrices are independent, with no data-path collective): each
rank runs the whole step, the timed region is bracketed by barriers, and rank 0 reports
the maximum time over ranks and the sum of matrices.  These tests check those host-side
pieces -- the barrier, max and sum helpers, and a real two-rank torchrun launch of the
reference arm, in which rank 0 alone prints the JSON line and the other rank exits 0."""
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


def _rank_main(rank, world, port, q):
    import importlib.util

    import torch.distributed as dist
    os.environ.update(MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port), RANK=str(rank), WORLD_SIZE=str(world), LOCAL_RANK=str(rank))
    dist.init_process_group("gloo", init_method="env://")
    spec = importlib.util.spec_from_file_location("bench_mod", os.path.join(ROOT, "bench.py"))
    bench = importlib.util.module_from_spec(spec)
    spec.loader.exec_module(bench)
    bench.barrier(dist)
    res = (bench.rank_env(), bench.allmax(dist, 1.5 + rank), bench.allsum(dist, 10.0 * (rank + 1)))
    bench.barrier(dist)
    dist.destroy_process_group()
    q.put((rank, res))


def test_gloo_helpers_two_ranks():
    import torch.multiprocessing as mp
    ctx = mp.get_context("spawn")
    q = ctx.Queue()
    port = free_port()
    procs = [ctx.Process(target=_rank_main, args=(r, 2, port, q)) for r in range(2)]
    for p in procs:
        p.start()
    out = dict(q.get(timeout=120) for _ in procs)
    for p in procs:
        p.join(timeout=60)
        assert p.exitcode == 0
    for r in range(2):
        env, mx, sm = out[r]
        assert env == (r, r, 2)
        assert mx == 2.5 and sm == 30.0


def test_reference_arm_two_ranks():
    """torchrun with two CPU ranks: one JSON line from rank 0, impl "reference", n_gpus 2"""
    pytest.importorskip("torch")
    cmd = [sys.executable, "-m", "torch.distributed.run", "--nnodes=1", "--nproc-per-node", "2", "--master-addr", "127.0.0.1",
           "--master-port", str(free_port()), os.path.join(ROOT, "bench.py"), "--impl", "reference", "--gpus", "2",
           "--steps", "1", "--warmup", "0", "--cpu-sample", "1"]
    env = dict(os.environ, OMP_NUM_THREADS="1")
    r = subprocess.run(cmd, cwd=ROOT, capture_output=True, text=True, timeout=600, env=env)
    assert r.returncode == 0, r.stderr[-2000:]
    lines = [l for l in r.stdout.splitlines() if l.startswith("{")]
    assert len(lines) == 1, r.stdout
    d = json.loads(lines[0])
    assert d["impl"] == "reference" and d["n_gpus"] == 2 and d["value"] > 0
    assert d["e2e"]["h2d_bytes_per_step"] == 0 and d["cpu_baseline"]["kind"] in ("port", "reference")
