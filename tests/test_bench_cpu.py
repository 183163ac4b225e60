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


def test_study_orders(monkeypatch):
    """bench.py --study: one run per grid side through run_to_tend and the
    order log2(e(h) / e(h/2)) between successive grids (run_to_tend faked
    here with errors of order 5)."""
    sys.path.insert(0, REPO)
    import argparse
    import aderdg
    import bench
    seen = []

    def fake(ad, cfg, ic, params, tend):
        seen.append((cfg.imax, cfg.N, cfg.limiter, cfg.precision, tend))
        e = 1e-3 * (32.0 / cfg.imax) ** 5
        return {"steps": cfg.imax, "tts_s": 1.0, "limited_cells_at_end": 0,
                "error_vs_exact": {"l1": e, "l2": 2 * e, "linf": 4 * e}}
    monkeypatch.setattr(bench, "run_to_tend", fake)
    args = argparse.Namespace(study="32,64,128,256", workload="euler_vortex", precision="fp64", N=0)
    out = bench.run_study(args, aderdg)
    assert seen == [(s, 4, 1, aderdg.FP64, 10.0) for s in (32, 64, 128, 256)]
    assert [g["side"] for g in out["grids"]] == [32, 64, 128, 256]
    assert "order_l1" not in out["grids"][0]
    for g in out["grids"][1:]:
        assert abs(g["order_l1"] - 5.0) < 1e-12 and abs(g["order_linf"] - 5.0) < 1e-12
