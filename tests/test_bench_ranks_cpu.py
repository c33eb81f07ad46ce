"""bench.py's multi-rank path on CPU (gloo, world size 2): each GPU runs an
independent replica, the timed region's length is the maximum over ranks
(reduce_max), the whole-job rate is ranks x units / that time
(whole_job_rate), and the CPU reference arm runs on rank 0 alone (other
ranks exit 0 without output)."""
import json
import os
import socket
import subprocess
import sys
from pathlib import Path

ROOT = Path(__file__).resolve().parent.parent

WORKER = r"""
import json, sys
sys.path.insert(0, {root!r})
import torch
import torch.distributed as dist
import bench
dist.init_process_group("gloo")
rank, ws = dist.get_rank(), dist.get_world_size()
slowest = bench.reduce_max(10.0 + 5.0 * rank, dist, torch)
print(json.dumps({{"rank": rank, "ws": ws, "max": slowest,
                   "rate": bench.whole_job_rate(1000.0, slowest, ws)}}))
dist.destroy_process_group()
"""


def free_port():
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def env_for(rank, ws, port):
    env = dict(os.environ, RANK=str(rank), WORLD_SIZE=str(ws), LOCAL_RANK=str(rank),
               MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port))
    env.pop("CUDA_VISIBLE_DEVICES", None)
    return env


def test_max_over_ranks_and_whole_job_rate():
    port, ws = free_port(), 2
    code = WORKER.format(root=str(ROOT))
    procs = [subprocess.Popen([sys.executable, "-c", code], env=env_for(r, ws, port), cwd=ROOT,
                              stdout=subprocess.PIPE, stderr=subprocess.PIPE, text=True) for r in range(ws)]
    outs = []
    for p in procs:
        out, err = p.communicate(timeout=120)
        assert p.returncode == 0, err[-2000:]
        outs.append(json.loads(out.strip().splitlines()[-1]))
    for o in outs:
        assert o["ws"] == 2 and o["max"] == 15.0  # the slower rank's time on every rank
        assert o["rate"] == 2 * 1000.0 / 15.0


def test_reference_arm_runs_on_rank_zero_only():
    r = subprocess.run([sys.executable, "bench.py", "--impl", "reference", "--gpus", "2", "--steps", "3",
                        "--warmup", "3"], env=env_for(1, 2, free_port()), cwd=ROOT,
                       capture_output=True, text=True, timeout=120)
    assert r.returncode == 0, r.stderr[-2000:]
    assert r.stdout.strip() == ""


def test_reference_arm_line():
    """The reference arm's JSON line on a small laminate: the keys the GPU
    arm's line carries, with its CPU baseline described and zero transfer
    bytes."""
    r = subprocess.run([sys.executable, "bench.py", "--impl", "reference", "--steps", "1", "--warmup", "3",
                        "--cpu-seconds", "1", "--nx", "40", "--ny", "40", "--nz", "8"],
                       env=env_for(0, 1, free_port()), cwd=ROOT, capture_output=True, text=True, timeout=300)
    assert r.returncode == 0, r.stderr[-2000:]
    line = json.loads(r.stdout.strip().splitlines()[-1])
    for key in ("impl", "metric", "value", "unit", "n_gpus", "steps", "warmup", "ms_per_step",
                "higher_is_better", "scaling", "dtype", "data", "config", "cpu_baseline", "e2e"):
        assert key in line, key
    assert line["impl"] == "reference" and line["value"] > 0 and line["higher_is_better"] is True
    cb = line["cpu_baseline"]
    assert cb["kind"] in ("reference", "port") and cb["cores"] >= 1 and cb["value"] == line["value"]
    assert cb["sample"]
    assert line["e2e"]["h2d_bytes_per_step"] == 0 and line["e2e"]["d2h_bytes_per_step"] == 0
    assert line["e2e"]["value"] == line["value"] and line["e2e"]["unit"] == line["unit"]
