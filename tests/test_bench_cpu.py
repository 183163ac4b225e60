"""The reference arm of bench.py (the FP64 CPU restatement on the host cores)
reports a value that follows from its own timing: value x ms_per_step / 1000
equals its DOF-updates per step."""
import json
import os
import subprocess
import sys

REPO = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def test_reference_arm_value_follows_from_its_timing():
    env = dict(os.environ)
    for k in ("WORLD_SIZE", "RANK", "LOCAL_RANK"):
        env.pop(k, None)
    r = subprocess.run([sys.executable, os.path.join(REPO, "bench.py"), "--impl", "reference", "--steps", "2",
                        "--warmup", "1"], capture_output=True, text=True, env=env, timeout=600)
    assert r.returncode == 0, r.stderr[-2000:]
    line = json.loads(r.stdout.strip().splitlines()[-1])
    assert line["impl"] == "reference" and line["value"] > 0
    per_step = line["value"] * line["ms_per_step"] / 1e3
    assert abs(per_step - line["dof_updates_per_step"]) <= 0.01 * line["dof_updates_per_step"]
    assert line["cpu_baseline"]["cores"] == (os.cpu_count() or 1)
