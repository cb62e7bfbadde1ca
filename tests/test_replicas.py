"""The N>1 path on CPU: replicas over torch.distributed with the gloo backend, world size 2.

The pass has no data-path collective (one independent solve per GPU), so the only cross-rank
operations are the bench's barrier and its max-over-ranks of the timed region.  These tests run
two real processes and check those operations, and that the reference arm works under torchrun
(rank 0 measures and prints, the other rank exits 0 without work).
"""
import json
import os
import socket
import subprocess
import sys
import textwrap

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def free_port() -> int:
    s = socket.socket()
    s.bind(("127.0.0.1", 0))
    port = s.getsockname()[1]
    s.close()
    return port


def test_ranks_barrier_and_max_gloo(tmp_path):
    pytest.importorskip("torch")
    port = free_port()
    script = textwrap.dedent(f"""
        import json, os, sys
        sys.path.insert(0, {ROOT!r})
        import bench
        r = bench.Ranks()
        assert r.world == 2 and r.backend == "gloo"
        r.barrier()
        m = r.max(1.5 + r.rank)
        r.barrier()
        with open(os.path.join({str(tmp_path)!r}, f"rank{{r.rank}}.json"), "w") as f:
            json.dump({{"rank": r.rank, "max": m}}, f)
        r.close()
    """)
    procs = []
    for rank in range(2):
        env = dict(os.environ, RANK=str(rank), LOCAL_RANK=str(rank), WORLD_SIZE="2", MASTER_ADDR="127.0.0.1",
                   MASTER_PORT=str(port), CUDA_VISIBLE_DEVICES="")
        procs.append(subprocess.Popen([sys.executable, "-c", script], env=env))
    for p in procs:
        assert p.wait(timeout=120) == 0
    for rank in range(2):
        with open(tmp_path / f"rank{rank}.json") as f:
            d = json.load(f)
        assert d["max"] == 2.5  # max over ranks of (1.5 + rank)


def test_reference_arm_under_torchrun_two_ranks():
    pytest.importorskip("torch")
    port = free_port()
    env = dict(os.environ, CUDA_VISIBLE_DEVICES="")
    cmd = [sys.executable, "-m", "torch.distributed.run", "--nnodes=1", "--nproc-per-node", "2", "--master-addr",
           "127.0.0.1", "--master-port", str(port), os.path.join(ROOT, "bench.py"), "--impl", "reference", "--gpus",
           "2", "--steps", "3", "--warmup", "3", "--n-ind", "400", "--n-snp", "3000", "--cpu-snps", "600"]
    r = subprocess.run(cmd, env=env, capture_output=True, text=True, timeout=300, cwd=ROOT)
    assert r.returncode == 0, r.stderr[-2000:]
    lines = [ln for ln in r.stdout.splitlines() if ln.startswith("{")]
    assert len(lines) == 1  # rank 0 alone prints
    d = json.loads(lines[0])
    assert d["impl"] == "reference" and d["n_gpus"] == 2 and d["value"] > 0
    assert d["cpu_baseline"]["kind"] == "port" and d["e2e"]["h2d_bytes_per_step"] == 0
