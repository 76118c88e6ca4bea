"""Multi-rank host logic of bench.py on CPU (gloo, world size 2).

The path has one grid per device, so N GPUs run N replicas; the reference
arm runs on rank 0 only and the other ranks exit 0 without output."""
import json
import os
import socket
import subprocess
import sys

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def _free_port():
    s = socket.socket()
    s.bind(("127.0.0.1", 0))
    port = s.getsockname()[1]
    s.close()
    return port


def test_reference_arm_two_ranks_prints_one_line():
    cmd = [sys.executable, "-m", "torch.distributed.run", "--nnodes=1", "--nproc-per-node=2",
           "--master-addr=127.0.0.1", f"--master-port={_free_port()}", os.path.join(ROOT, "bench.py"),
           "--impl", "reference", "--gpus", "2", "--grid", "64", "--steps", "2", "--warmup", "1"]
    env = dict(os.environ, OMP_NUM_THREADS="2")
    r = subprocess.run(cmd, capture_output=True, text=True, timeout=300, env=env, cwd=ROOT)
    assert r.returncode == 0, r.stderr[-3000:]
    lines = [ln for ln in r.stdout.splitlines() if ln.startswith("{")]
    assert len(lines) == 1
    d = json.loads(lines[0])
    assert d["impl"] == "reference" and d["n_gpus"] == 2
    assert d["unit"] == "grid-point stage updates/s" and d["value"] > 0
    assert d["cpu_baseline"]["kind"] in ("port", "reference")
    assert d["e2e"]["h2d_bytes_per_step"] == 0


def test_max_over_ranks_reduction_gloo(tmp_path):
    """bench.py's timing reduction (max_over_ranks: an all_reduce MAX of the ranks' elapsed
    times) across two gloo ranks, and its one-rank form without a process group."""
    code = r'''
import sys, torch.distributed as dist
sys.path.insert(0, sys.argv[1])
import bench
assert bench.max_over_ranks(7.5, None, "cpu") == 7.5
dist.init_process_group("gloo")
r = dist.get_rank()
assert bench.max_over_ranks(10.0 + 5.0 * r, dist, "cpu") == 15.0
assert bench.max_over_ranks(3.0 - r, dist, "cpu") == 3.0
if r == 0:
    print("OK")
dist.destroy_process_group()
'''
    path = tmp_path / "maxreduce_child.py"
    path.write_text(code)
    cmd = [sys.executable, "-m", "torch.distributed.run", "--nnodes=1", "--nproc-per-node=2",
           "--master-addr=127.0.0.1", f"--master-port={_free_port()}", str(path), ROOT]
    r = subprocess.run(cmd, capture_output=True, text=True, timeout=120)
    assert r.returncode == 0, r.stderr[-2000:]
    assert "OK" in r.stdout
