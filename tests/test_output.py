"""Output and error analysis: the device cell averages (and their primitive
variables) are write_data's field in the reference's summation order; the VTK
files follow write_data / plot_troubled_cells; the error norms reproduce
analyze_soln and measure the error against exact solutions; the C++ driver
writes the files every WriteInterval steps and prints analyze_soln."""
import subprocess

import numpy as np
import pytest

import aderdg
from test_driver import EULER_DMR, _write

pytestmark = pytest.mark.gpu


def _averages_reference_order(uh, cfg):
    """Euler/write_data.f90:21-29 in Python loops: Q(v) += w(ii) w(jj) uh(v, ii, jj)."""
    P, V = cfg.N + 1, cfg.nvar
    w = aderdg.operator(cfg.N, aderdg.OP_W)
    u = uh.reshape(cfg.cells, P * P, V)
    out = np.zeros((cfg.cells, V))
    for c in range(cfg.cells):
        for v in range(V):
            q = 0.0
            for jj in range(P):
                for ii in range(P):
                    q = q + w[ii] * w[jj] * u[c, ii + P * jj, v]
            out[c, v] = q
    return out


def test_cell_averages_and_primitives(gpu_lib):
    cfg, ic, params, tend = aderdg.workloads.make("euler_rp2d", side=6, N=3)
    s = aderdg.Solver(cfg)
    s.initial_condition(ic, params)
    t = 0.0
    for _ in range(2):
        t, _, _ = s.step(t, tend)
    uh, _ = s.download()
    Q = _averages_reference_order(uh, cfg)
    assert np.array_equal(s.cell_averages(primitive=False), Q)
    g = cfg.gamma
    prim = np.empty_like(Q)
    for c in range(cfg.cells):
        q = Q[c]
        prim[c] = (q[0], q[1] / q[0], q[2] / q[0], (g - 1.0) * (q[3] - 0.5 * (q[1] ** 2 + q[2] ** 2) / q[0]))
    assert np.array_equal(s.cell_averages(primitive=True), prim)
    s.close()


def test_batch_cell_averages_equal_solver(gpu_lib):
    cfg, ic, params, tend = aderdg.workloads.make("bn_cylinder", side=10, N=2)
    s = aderdg.Solver(cfg)
    s.initial_condition(ic, params)
    b = aderdg.Batch(cfg.system, cfg.N, cfg.precision, 1, capacity_units=512, max_instances=2)
    slot = b.admit_ic(cfg, ic, params, tend, 0)
    t = 0.0
    for _ in range(3):
        t, _, _ = s.step(t, tend)
    b.launch(3)
    b.sync()
    assert np.array_equal(b.cell_averages(slot), s.cell_averages())
    b.close()
    s.close()


def test_error_norms(gpu_lib):
    # at t = 0 against the field it was set from: exactly zero (analyze_soln's number)
    cfg, ic, params, tend = aderdg.workloads.make("euler_vortex", side=16, N=3)
    s = aderdg.Solver(cfg)
    s.initial_condition(ic, params)
    assert s.error_norms(ic, params) == (0.0, 0.0, 0.0)
    s.close()
    # advection-diffusion with the fused flux against the exact translated, damped wave:
    # the error falls with the degree
    errs = []
    for N in (2, 3, 4):
        cfg, ic, params, tend = aderdg.workloads.make("ad_sine", side=8, N=N, ad_flux_mode=1)
        s = aderdg.Solver(cfg)
        s.initial_condition(ic, params)
        t, _ = s.run(0.0, 0.05, 100000)
        assert t == 0.05
        errs.append(s.error_norms(ic, params)[2])
        s.close()
    assert errs[0] > errs[1] > errs[2] and errs[2] < 1e-4, errs


def test_vtk_files(tmp_path, gpu_lib):
    cfg, ic, params, tend = aderdg.workloads.make("euler_rp2d", side=5, N=2)
    s = aderdg.Solver(cfg)
    s.initial_condition(ic, params)
    t, _, _ = s.step(0.0, tend)
    wh = s.cell_averages()
    path = tmp_path / "out.vtk"
    aderdg.output.write_vtk(str(path), cfg, wh, t)
    lines = path.read_text().splitlines()
    assert lines[3] == "DATASET STRUCTURED_GRID" and lines[7] == "DIMENSIONS     5    5    1"
    k = lines.index("SCALARS Density double 1")
    dens = [float(x) for x in lines[k + 2:k + 2 + cfg.cells]]
    assert np.allclose(dens, wh[:, 0], rtol=1e-6, atol=0)
    rec = s.get(aderdg.A_RECOMPUTE)
    tpath = tmp_path / "tc.vtk"
    aderdg.output.write_troubled_cells_vtk(str(tpath), cfg, rec, t)
    tl = tpath.read_text().splitlines()
    assert tl[3] == "DATASET UNSTRUCTURED_GRID"
    k = tl.index("SCALARS TCells double 1")
    vals = [float(x) for x in tl[k + 2:]]
    assert len(vals) == cfg.cells and set(vals) <= {0.0, 1.0, 2.0}
    s.close()


def test_driver_writes_vtk_and_analyzes(tmp_path, gpu_lib):
    ini = _write(tmp_path, "params.ini", EULER_DMR.replace("100     ! output interval", "2       ! output interval"))
    base = str(tmp_path / "dmr")
    r = subprocess.run([aderdg.builder.DRIVER_PATH, "euler", ini, "--max-steps", "4", "--quiet", "--vtk", base,
                        "--analyze"], capture_output=True, text=True, timeout=300)
    assert r.returncode == 0, r.stderr
    for k in (0, 2, 4):
        assert (tmp_path / ("dmr-%08d.vtk" % k)).exists()
        assert (tmp_path / ("Tcells-%08d.vtk" % k)).exists()
    err = float(r.stdout.strip().splitlines()[-1])
    assert err > 0.0
