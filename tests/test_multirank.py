"""The multi-rank path of bench.py on the CPU: two gloo ranks reduce the timing (the maximum of the elapsed
time, the sum of the attempts, as every rank runs an independent replica); the GPU arm's whole multi-rank
path with the engine replaced by a host-side stand-in (tests/multirank_bench_runner.py); `--gpus 2`
without torchrun spawning its own ranks; and the reference arm under torch.distributed.run, where rank 0
alone measures and prints one line and the other rank exits cleanly."""
import json
import os
import socket
import subprocess
import sys
import tempfile

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


def test_gpu_arm_aggregates_two_ranks_with_distinct_seeds():
    out = tempfile.mkdtemp(prefix="ppmr_")
    cmd = [sys.executable, "-m", "torch.distributed.run", "--nnodes=1", "--nproc-per-node", "2", "--master-addr", "127.0.0.1", "--master-port",
           str(_free_port()), os.path.join("tests", "multirank_bench_runner.py"), "--gpus", "2", "--steps", "4", "--warmup", "3",
           "--no-e2e", "--no-learned", "--no-cpu-baseline", "--tune-sweeps", "0", "--roofline-sweeps", "1"]
    p = subprocess.run(cmd, cwd=ROOT, capture_output=True, text=True, timeout=600, env=dict(os.environ, PP_FAKE_OUT=out))
    assert p.returncode == 0, p.stderr[-3000:]
    lines = [l for l in p.stdout.splitlines() if l.startswith("{")]
    assert len(lines) == 1, p.stdout[-2000:]
    d = json.loads(lines[0])
    # rank r: (1000 + r) attempts per sweep, 0.5 (1 + r) ms per sweep; value = all attempts / slowest rank
    assert d["n_gpus"] == 2 and d["steps"] == 4 and d["scaling"] == "weak"
    assert abs(d["value"] - (4 * 1000 + 4 * 1001) / 0.004) < 1e-6 * d["value"]
    assert abs(d["ms_per_step"] - 1.0) < 1e-9
    seen = [json.load(open(os.path.join(out, "rank%d.json" % r))) for r in (0, 1)]
    assert [s["device"] for s in seen] == [0, 1]
    assert seen[0]["engine_seeds"] != seen[1]["engine_seeds"] and seen[0]["generate_seeds"] != seen[1]["generate_seeds"]


def test_gpus_flag_without_torchrun_spawns_its_ranks():
    out = tempfile.mkdtemp(prefix="ppmr_")
    env = {k: v for k, v in os.environ.items() if k not in ("WORLD_SIZE", "RANK", "LOCAL_RANK")}
    env["PP_FAKE_OUT"] = out
    cmd = [sys.executable, os.path.join("tests", "multirank_bench_runner.py"), "--gpus", "2", "--steps", "2", "--warmup", "3",
           "--no-e2e", "--no-learned", "--no-cpu-baseline", "--tune-sweeps", "0", "--roofline-sweeps", "1"]
    p = subprocess.run(cmd, cwd=ROOT, capture_output=True, text=True, timeout=600, env=env)
    assert p.returncode == 0, p.stderr[-3000:]
    lines = [l for l in p.stdout.splitlines() if l.startswith("{")]
    assert len(lines) == 1 and json.loads(lines[0])["n_gpus"] == 2
