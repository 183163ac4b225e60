"""The C++ driver (restatement of main.f90 over the C ABI) reads params.ini
files in the reference's positional formats and runs the loop; on the GPU its
final state must equal the Python path's for the same configuration."""
import os
import subprocess

import numpy as np
import pytest

import aderdg

EULER_DMR = """1.4     ! ratio of specific heats
48      ! cells in x
12      ! cells in y
0.0     ! x left
0.0     ! y bottom
4.0     ! x right
1.0     ! y top
1       ! left boundary
1       ! right boundary
1       ! bottom boundary
1       ! top boundary
11      ! initial condition
0.2     ! end time
100     ! output interval
"""

BN_RP = """1.4     ! gamma solid
1.4     ! gamma gas
0.0     ! pi solid
0.0     ! pi gas
40      ! cells in x
4       ! cells in y
-0.5    ! x left
-0.05   ! y bottom
0.5     ! x right
0.05    ! y top
1       ! left
1       ! right
1       ! bottom
1       ! top
3       ! initial condition type
0.1     ! end time
10000   ! output interval
N = 3
"""

AD = """1.0     ! cx
0.5     ! cy
0.01    ! diffusion
16      ! cells in x
16      ! cells in y
0.0
0.0
1.0
1.0
1.0     ! end time
3       ! left
3       ! right
3       ! bottom
3       ! top
500     ! output interval
N = 3
ic = sine
"""


def _driver():
    return aderdg.builder.DRIVER_PATH


def _write(tmp_path, name, text):
    p = tmp_path / name
    p.write_text(text)
    return str(p)


def test_driver_rejects_bad_params_without_touching_the_gpu(tmp_path, gpu_lib):
    bad = _write(tmp_path, "bad.ini", "1.4\n48\n")
    r = subprocess.run([_driver(), "euler", bad], capture_output=True, text=True)
    assert r.returncode == 2 and "too few fields" in r.stderr
    r = subprocess.run([_driver(), "euler", _write(tmp_path, "ext.ini", EULER_DMR + "bogus = 1\n")],
                       capture_output=True, text=True)
    assert r.returncode == 2 and "unknown extension key" in r.stderr
    r = subprocess.run([_driver(), "mhd", bad], capture_output=True, text=True)
    assert r.returncode == 2


def _read_dump(path):
    with open(path, "rb") as fh:
        steps = np.frombuffer(fh.read(8), dtype=np.int64)[0]
        t = np.frombuffer(fh.read(8), dtype=np.float64)[0]
        uh = np.frombuffer(fh.read(), dtype=np.float64)
    return int(steps), float(t), uh


CASES = [
    ("euler", EULER_DMR, aderdg.Config(system=aderdg.SYS_EULER, N=1, imax=48, jmax=12, xr=(4.0, 1.0), bc_mode=1),
     aderdg.IC_EULER_DMR, (), 0.2),
    ("bn", BN_RP, aderdg.Config(system=aderdg.SYS_BN, N=3, imax=40, jmax=4, xl=(-0.5, -0.05), xr=(0.5, 0.05)),
     aderdg.IC_BN_RP1D, (3.0, 0.0), 0.1),
    ("ad", AD, aderdg.Config(system=aderdg.SYS_ADVDIFF, N=3, imax=16, jmax=16, bc=(3, 3, 3, 3), cx=1.0, cy=0.5,
                             a=0.01, limiter=0), aderdg.IC_AD_SINE, (1.0,), 1.0),
]


@pytest.mark.gpu
@pytest.mark.parametrize("sysname,text,cfg,ic,params,tend", CASES)
def test_driver_matches_python_path(tmp_path, gpu_lib, sysname, text, cfg, ic, params, tend):
    ini = _write(tmp_path, "params.ini", text)
    out = str(tmp_path / "uh.bin")
    r = subprocess.run([_driver(), sysname, ini, "--max-steps", "4", "--quiet", "--dump", out], capture_output=True,
                       text=True, timeout=300)
    assert r.returncode == 0, r.stderr
    steps, t, uh_drv = _read_dump(out)
    assert steps == 4
    uh, lh = aderdg.project_initial_condition(cfg, ic, params)
    s = aderdg.Solver(cfg)
    s.upload(uh)
    if cfg.limiter and cfg.system != aderdg.SYS_ADVDIFF:
        s.init_limiter(lh)
    tt = 0.0
    for _ in range(4):
        tt, _, _ = s.step(tt, tend)
    ug, _ = s.download()
    assert tt == t
    assert np.array_equal(ug, uh_drv)
    # the phase-by-phase loop differs from the fused one only by rounding
    out2 = str(tmp_path / "uh2.bin")
    r = subprocess.run([_driver(), sysname, ini, "--max-steps", "4", "--quiet", "--phases", "--dump", out2],
                       capture_output=True, text=True, timeout=300)
    assert r.returncode == 0, r.stderr
    _, t2, uh_ph = _read_dump(out2)
    assert abs(t2 - t) <= 1e-14 * max(1.0, t)
    assert np.abs(uh_ph - uh_drv).sum() <= 1e-11 * np.abs(uh_drv).sum()
