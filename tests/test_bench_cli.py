"""bench.py's command line on the CPU: `--gpus 2` started as one process
runs again as two ranks under torch.distributed.run, and rank 0 alone
prints the line of the reference arm (the oracle's CPU solve), which reports
both ranks."""

import json
import os
import subprocess
import sys

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def _run(args):
    env = dict(os.environ)
    env.pop("WORLD_SIZE", None)
    p = subprocess.run([sys.executable, os.path.join(ROOT, "bench.py")] + args,
                       capture_output=True, text=True, timeout=300, env=env, cwd=ROOT)
    assert p.returncode == 0, p.stderr[-2000:]
    lines = [ln for ln in p.stdout.splitlines() if ln.startswith("{")]
    return [json.loads(ln) for ln in lines]


def test_reference_arm_two_ranks():
    out = _run(["--impl", "reference", "--gpus", "2", "--size", "48", "--steps", "2",
                "--warmup", "1"])
    assert len(out) == 1                      # rank 0 alone prints
    rec = out[0]
    assert rec["impl"] == "reference" and rec["n_gpus"] == 2
    assert rec["steps"] == 2 and rec["warmup"] == 1
    assert rec["config"]["parallelism"] == "replicas x2"
    assert rec["cpu_baseline"]["kind"] == "port"
    assert rec["e2e"]["h2d_bytes_per_step"] == 0
    # every step is a whole solve to the gap
    assert rec["iters_to_gap"] > 0 and abs(rec["final_relgap"]) < 1e-4


def test_reference_arm_one_rank():
    out = _run(["--impl", "reference", "--size", "48", "--steps", "1", "--warmup", "1"])
    assert len(out) == 1 and out[0]["n_gpus"] == 1
