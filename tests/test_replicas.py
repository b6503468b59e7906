"""The N > 1 path of bench.py on CPU with gloo, world size 2: the path does
not shard (replicas only), so ranks only meet in the barrier and the
max / sum reductions of their timings and counts; the reference arm runs on
rank 0 alone and prints one line."""
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


def _worker(rank, port, out):
    os.environ.update(MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port), WORLD_SIZE="2", RANK=str(rank))
    sys.path.insert(0, ROOT)
    import bench
    r, ws = bench.dist()
    bench.barrier(ws)
    out[rank] = (r, ws, bench.allreduce_sum(float(rank + 1), ws), bench.allreduce_max(10.0 * (rank + 1), ws))


def test_reductions_over_two_gloo_ranks():
    torch = pytest.importorskip("torch")
    mp = torch.multiprocessing.get_context("spawn")
    out = mp.Manager().dict()
    port = free_port()
    ps = [mp.Process(target=_worker, args=(r, port, out)) for r in (0, 1)]
    for p in ps:
        p.start()
    for p in ps:
        p.join(120)
        assert p.exitcode == 0
    assert out[0] == (0, 2, 3.0, 20.0) and out[1] == (1, 2, 3.0, 20.0)


def test_reference_arm_prints_once_under_torchrun():
    pytest.importorskip("torch")
    cmd = [sys.executable, "-m", "torch.distributed.run", "--nnodes=1", "--nproc-per-node", "2",
           "--master-addr", "127.0.0.1", "--master-port", str(free_port()), "bench.py", "--impl", "reference",
           "--gpus", "2", "--steps", "1", "--warmup", "1", "--cells", "8", "--ppc", "1"]
    r = subprocess.run(cmd, cwd=ROOT, capture_output=True, text=True, timeout=600)
    assert r.returncode == 0, r.stderr[-2000:]
    lines = [l for l in r.stdout.splitlines() if l.startswith("{")]
    assert len(lines) == 1
    d = json.loads(lines[0])
    assert d["impl"] == "reference" and d["value"] > 0 and d["e2e"]["h2d_bytes_per_step"] == 0
