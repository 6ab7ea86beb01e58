"""bench.py --gpus N starts N ranks itself (torch.distributed.run) when it is not
already under torchrun, and the multi-rank path (barriers, max over ranks, rank 0's one
JSON line with n_gpus = N) runs on the CPU with --dry-run (gloo, the FP32 oracle
standing in for the GPU step)."""
import json
import os
import subprocess
import sys

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def test_two_rank_dry_run_prints_one_line_with_two_gpus():
    env = {k: v for k, v in os.environ.items() if k not in ("WORLD_SIZE", "RANK", "LOCAL_RANK", "MASTER_ADDR",
                                                             "MASTER_PORT")}
    r = subprocess.run([sys.executable, os.path.join(ROOT, "bench.py"), "--gpus", "2", "--dry-run", "--steps", "2",
                        "--warmup", "3"], cwd=ROOT, env=env, capture_output=True, text=True, timeout=600)
    assert r.returncode == 0, r.stderr[-3000:]
    lines = [ln for ln in r.stdout.splitlines() if ln.strip().startswith("{")]
    assert len(lines) == 1, r.stdout
    d = json.loads(lines[0])
    assert d["n_gpus"] == 2 and d["steps"] == 2 and d["warmup"] == 3 and d["value"] > 0
    assert d["scaling"] == "weak"
