"""The multi-rank path of bench.py on the CPU: two gloo ranks reduce the timing (the maximum of the elapsed
time, the sum of the attempts, as every rank runs an independent replica), and the reference arm under
torch.distributed.run, where rank 0 alone measures and prints one line and the other rank exits cleanly."""
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


def _worker(rank, port, out):
    os.environ.update(MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port), RANK=str(rank), WORLD_SIZE="2", LOCAL_RANK=str(rank))
    if ROOT not in sys.path:
        sys.path.insert(0, ROOT)
    import bench

    ws, r, local, dist = bench.dist_setup()
    mx = bench.allreduce(dist, 1.5 * (rank + 1), bench._max_op(dist))
    sm = bench.allreduce(dist, float(rank + 1), bench._sum_op(dist))
    bench.barrier(dist)
    out[rank] = (ws, r, local, mx, sm)
    dist.destroy_process_group()


def test_timing_reductions_over_two_gloo_ranks():
    import torch.multiprocessing as mp

    mgr = mp.Manager()
    out = mgr.dict()
    mp.spawn(_worker, args=(_free_port(), out), nprocs=2, join=True)
    assert out[0] == (2, 0, 0, 3.0, 3.0) and out[1] == (2, 1, 1, 3.0, 3.0)


def test_reference_arm_under_torchrun():
    cmd = [sys.executable, "-m", "torch.distributed.run", "--nnodes=1", "--nproc-per-node", "2", "--master-addr", "127.0.0.1", "--master-port",
           str(_free_port()), "bench.py", "--impl", "reference", "--workload", "c1", "--steps", "1", "--warmup", "3", "--gpus", "2"]
    p = subprocess.run(cmd, cwd=ROOT, capture_output=True, text=True, timeout=600)
    assert p.returncode == 0, p.stderr[-2000:]
    lines = [l for l in p.stdout.splitlines() if l.startswith("{")]
    assert len(lines) == 1
    d = json.loads(lines[0])
    assert d["impl"] == "reference" and d["n_gpus"] == 2 and d["value"] > 0 and d["cpu_baseline"]["cores"] >= 1
