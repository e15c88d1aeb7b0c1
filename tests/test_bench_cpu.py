"""bench.py host logic without a GPU: the max-over-ranks reduction on two gloo
ranks, the CPU reference arm's JSON line, and the algorithmic-byte model."""
import json
import os
import subprocess
import sys

import pytest

from conftest import ROOT


def _worker(rank, world, port, q):
    os.environ.update(MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port), RANK=str(rank),
                      WORLD_SIZE=str(world))
    sys.path.insert(0, ROOT)
    import torch.distributed as dist
    import bench
    dist.init_process_group("gloo", rank=rank, world_size=world)
    t = bench.reduce_max(dist, 10.0 + rank)
    bench.barrier(dist)
    q.put((rank, t))
    dist.destroy_process_group()


def test_reduce_max_two_gloo_ranks():
    import multiprocessing as mp
    import socket
    s = socket.socket()
    s.bind(("127.0.0.1", 0))
    port = s.getsockname()[1]
    s.close()
    ctx = mp.get_context("spawn")
    q = ctx.Queue()
    ps = [ctx.Process(target=_worker, args=(r, 2, port, q)) for r in range(2)]
    for p in ps:
        p.start()
    for p in ps:
        p.join(120)
    out = dict(q.get(timeout=5) for _ in range(2))
    assert out == {0: 11.0, 1: 11.0}


def test_reference_arm_line():
    from oracle import orc
    if not orc.reference_available("fierro_ref_fast"):
        from oracle import build_ref
        if build_ref.build_reference() is None:
            pytest.skip("reference sources unavailable")
    p = subprocess.run([sys.executable, os.path.join(ROOT, "bench.py"), "--impl", "reference", "--cpu-n", "12",
                        "--steps", "2", "--warmup", "1"], capture_output=True, text=True, timeout=300)
    assert p.returncode == 0, p.stderr
    line = json.loads(p.stdout.strip().splitlines()[-1])
    assert line["impl"] == "reference"
    assert line["value"] > 0 and line["unit"] == "element-cycles/s"
    assert line["cpu_baseline"]["kind"] == "reference" and line["cpu_baseline"]["cores"] >= 1
    assert line["e2e"]["h2d_bytes_per_step"] == 0


def test_reference_arm_two_ranks_prints_once():
    """Under torchrun with two ranks (gloo here) rank 0 alone runs the reference
    arm and prints its line; rank 1 exits 0 without output."""
    import socket
    from oracle import orc
    if not orc.reference_available("fierro_ref_fast"):
        from oracle import build_ref
        if build_ref.build_reference() is None:
            pytest.skip("reference sources unavailable")
    s = socket.socket()
    s.bind(("127.0.0.1", 0))
    port = s.getsockname()[1]
    s.close()
    p = subprocess.run([sys.executable, "-m", "torch.distributed.run", "--nnodes=1", "--nproc-per-node", "2",
                        "--master-addr", "127.0.0.1", "--master-port", str(port),
                        os.path.join(ROOT, "bench.py"), "--impl", "reference", "--gpus", "2", "--cpu-n", "8",
                        "--steps", "1", "--warmup", "0"], capture_output=True, text=True, timeout=300)
    assert p.returncode == 0, p.stderr[-2000:]
    lines = [ln for ln in p.stdout.splitlines() if ln.startswith("{")]
    assert len(lines) == 1, p.stdout
    assert json.loads(lines[0])["impl"] == "reference"


def test_alg_bytes_model():
    import bench
    n = 64
    nn, ne = (n + 1) ** 3, n ** 3
    from fierro_gb300 import problems
    nnz = bench.solver_neighbor_count(problems.sedov(n))
    assert nnz == (3 * n - 2) ** 3 - n ** 3
    for k in ("k_force", "k_node", "k_elem"):
        b = bench.alg_bytes(k, nn, ne, nnz)
        assert 300 * ne < b < 900 * ne
