"""The N > 1 path on the CPU (gloo, world size 2).  The path shards as replicas, with no
collective in the data path; these tests cover the bench's whole-job rate over ranks (the
slowest rank's time, the sum of the ranks' rays) and its reference arm, which rank 0 alone runs
while the other ranks exit 0 without work."""
import json
import os
import socket
import subprocess
import sys

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))

RATE_SCRIPT = r'''
import json, os, sys
sys.path.insert(0, sys.argv[1])
import torch.distributed as dist
dist.init_process_group("gloo")
rank, world = dist.get_rank(), dist.get_world_size()
import bench
ms, units = [12.5, 20.0][rank], [1000.0, 3000.0][rank]
out = bench.job_rate(ms, units, world, "cpu")
with open(os.path.join(sys.argv[2], f"rank{rank}.json"), "w") as f:
    json.dump(out, f)
dist.barrier()
dist.destroy_process_group()
'''


def _port():
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def _torchrun(args, timeout):
    cmd = [sys.executable, "-m", "torch.distributed.run", "--nnodes=1", "--nproc-per-node=2",
           "--master-addr=127.0.0.1", f"--master-port={_port()}"] + args
    env = dict(os.environ, OMP_NUM_THREADS="1")
    return subprocess.run(cmd, cwd=ROOT, env=env, capture_output=True, text=True, timeout=timeout)


def test_job_rate_over_two_ranks(tmp_path):
    script = tmp_path / "rate.py"
    script.write_text(RATE_SCRIPT)
    r = _torchrun([str(script), ROOT, str(tmp_path)], timeout=300)
    assert r.returncode == 0, r.stderr[-2000:]
    for rank in range(2):
        ms_max, total, rate = json.loads((tmp_path / f"rank{rank}.json").read_text())
        assert ms_max == 20.0 and total == 4000.0 and rate == 4000.0 / 0.02


def test_reference_arm_runs_on_rank_zero_only():
    r = _torchrun(["bench.py", "--impl", "reference", "--steps", "1", "--warmup", "0", "--cpu-sample", "4096"],
                  timeout=600)
    assert r.returncode == 0, r.stderr[-2000:]
    lines = [json.loads(x) for x in r.stdout.splitlines() if x.startswith("{")]
    assert len(lines) == 1   # rank 1 printed nothing
    line = lines[0]
    assert line["impl"] == "reference" and line["n_gpus"] == 2 and line["value"] > 0
    assert line["cpu_baseline"]["kind"] in ("port", "reference") and line["e2e"]["h2d_bytes_per_step"] == 0
