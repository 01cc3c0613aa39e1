"""Multi-process (world_size 2, gloo, CPU) coverage of the N > 1 bench path.

Pairs are independent, so N GPUs run N weak-scaling replicas with no data-path
collective; the only cross-rank step is the timing reduction (slowest rank,
units summed), and under torchrun the reference arm runs on rank 0 alone.
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


def _reduce_worker(rank, world, port, q):
    os.environ.update(MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port))
    import torch.distributed as dist
    sys.path.insert(0, ROOT)
    import bench
    dist.init_process_group("gloo", rank=rank, world_size=world)
    try:
        # rank r: 10 + r ms for 1000 * (r + 1) cells; e2e 0.5 + r s
        out = bench.reduce_over_ranks(10.0 + rank, 1000 * (rank + 1), 0.5 + rank,
                                      1000 * (rank + 1), world)
        q.put((rank, out))
    finally:
        dist.destroy_process_group()


def test_reduce_over_ranks_gloo():
    world = 2
    ctx = mp.get_context("spawn")
    q = ctx.Queue()
    port = _free_port()
    procs = [ctx.Process(target=_reduce_worker, args=(r, world, port, q)) for r in range(world)]
    for p in procs:
        p.start()
    got = dict(q.get(timeout=120) for _ in range(world))
    for p in procs:
        p.join(60)
        assert p.exitcode == 0
    for r in range(world):
        ms, cells, e2e_s, e2e_cells = got[r]
        assert ms == 11.0 and cells == 3000.0
        assert e2e_s == 1.5 and e2e_cells == 3000.0


def test_reference_arm_under_torchrun_two_ranks():
    pytest.importorskip("numpy")
    port = _free_port()
    cmd = [sys.executable, "-m", "torch.distributed.run", "--nnodes=1", "--nproc-per-node", "2",
           "--master-addr", "127.0.0.1", "--master-port", str(port), "bench.py", "--impl",
           "reference", "--gpus", "2", "--config", "0", "--steps", "1", "--warmup", "1",
           "--cpu-sample", "64"]
    env = dict(os.environ, OMP_NUM_THREADS="1")
    r = subprocess.run(cmd, cwd=ROOT, capture_output=True, text=True, timeout=300, env=env)
    assert r.returncode == 0, r.stderr[-2000:]
    lines = [ln for ln in r.stdout.splitlines() if ln.startswith("{")]
    assert len(lines) == 1, r.stdout  # rank 0 alone prints
    d = json.loads(lines[0])
    assert d["impl"] == "reference" and d["n_gpus"] == 2 and d["value"] > 0
    assert d["cpu_baseline"]["kind"] == "port"
    assert d["e2e"]["h2d_bytes_per_step"] == 0
    # the arm maps the oracle's library only, never the GPU path's
    libs = d["repo_libraries_loaded"]
    if libs is not None:
        assert libs and all(x.startswith("oracle" + os.sep) for x in libs), libs
