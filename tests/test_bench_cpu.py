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


def test_clock_summary_flags_throttling():
    """The clocks record of a timed region: median SM clock, the maximum, and
    every throttle reason seen active (the fields of nvidia-smi's query)."""
    sys.path.insert(0, REPO)
    import bench
    c = bench.ClockSampler()
    assert c.summary()["reasons"] == ["nvidia-smi unavailable"]
    row = "0, {sm}, 2070, 900.0, 0x0, {hw}, Not Active, Not Active, {cap}"
    rows = ((2070, "Not Active", "Not Active"), (1980, "Not Active", "Active"), (2070, "Active", "Not Active"))
    for sm, hw, cap in rows:
        c.samples.append([x.strip() for x in row.format(sm=sm, hw=hw, cap=cap).split(",")])
    s = c.summary()
    assert s["sm_mhz"] == 2070.0 and s["sm_max_mhz"] == 2070.0 and s["samples"] == 3
    assert s["reasons"] == ["hw_slowdown", "sw_power_cap"]
    c.samples = [[x.strip() for x in row.format(sm="[N/A]", hw="Not Active", cap="Not Active").split(",")]]
    assert c.summary()["sm_mhz"] is None


def test_error_summary():
    """error_vs_fp64: per-request relative errors and troubled-cell counts."""
    sys.path.insert(0, REPO)
    import bench
    errs = [dict(rel_l1=1e-7 * k, rel_linf=1e-6 * k, limited=10 + (k == 3), limited_fp64=10, mask_diff=int(k == 3))
            for k in range(1, 5)]
    s = bench._err_stats(errs)
    assert s["requests"] == 4 and s["max_l1"] == 4e-7 and s["max_linf"] == 4e-6
    assert abs(s["median_l1"] - 2.5e-7) < 1e-20
    assert s["limited_cells_fp64"] == 40 and s["mask_disagreements"] == 1
    assert abs(s["max_count_diff_pct"] - 10.0) < 1e-12 and abs(s["total_count_diff_pct"] - 2.5) < 1e-12


def test_traffic_from_the_committed_table():
    """roofline.traffic: the committed per-(system, N) bytes per unit times the
    units; None when a group has no capture."""
    sys.path.insert(0, REPO)
    import bench
    with open(os.path.join(REPO, "profiles", "traffic.json")) as fh:
        tr = json.load(fh)
    per = tr["k_subcell_bytes_per_listed_cell"]["fp32"]
    units = {(1, 3): 100, (2, 3): 7}
    tot, lim = bench._traffic(units, "k_subcell_bytes_per_listed_cell", "fp32")
    assert abs(tot - (100 * per["1_3"] + 7 * per["2_3"])) < 1e-6 and "FP64 pipe" in lim
    assert bench._traffic({(2, 9): 1}, "k_subcell_bytes_per_listed_cell", "fp32")[0] is None
    for key in ("k_predictor_bytes_per_dof", "k_subcell_bytes_per_listed_cell"):
        for s in (1, 2):
            for n in (2, 3, 4, 5):
                assert tr[key]["fp32"]["%d_%d" % (s, n)] > 0, (key, s, n)
