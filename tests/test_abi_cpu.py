"""CPU-side checks of the C-ABI library: it loads, exports every entry point
declared in include/aderdg_gpu.h, builds operators and initial fields that are
bit-identical to the oracle's, and rejects bad configurations before touching
the GPU.  No kernel runs here."""
import ctypes
import dataclasses
import os
import re

import numpy as np
import pytest

import aderdg
import pyoracle as po

from conftest import REPO
from helpers import oracle_config


def header_functions():
    text = open(os.path.join(REPO, "include", "aderdg_gpu.h")).read()
    text = re.sub(r"/\*.*?\*/", "", text, flags=re.S)
    return sorted(set(re.findall(r"\b(aderdg_[a-z_0-9]+)\s*\(", text)))


def test_library_exports_every_declared_symbol(gpu_lib):
    names = header_functions()
    assert len(names) >= 25
    for n in names:
        assert hasattr(gpu_lib, n), n
    assert set(aderdg.EXPORTED) <= set(names)


OPS = [(aderdg.OP_XI, po.OP_XI), (aderdg.OP_W, po.OP_W), (aderdg.OP_KXI, po.OP_KXI), (aderdg.OP_DUDX, po.OP_DUDX),
       (aderdg.OP_IK1, po.OP_IK1), (aderdg.OP_F0, po.OP_F0), (aderdg.OP_FL, po.OP_FL), (aderdg.OP_FR, po.OP_FR),
       (aderdg.OP_UH2LIM, po.OP_UH2LIM), (aderdg.OP_LIM2UH, po.OP_LIM2UH), (aderdg.OP_UH2LOB, po.OP_UH2LOB),
       (aderdg.OP_XILIMBARY, po.OP_XILIMBARY)]


@pytest.mark.parametrize("N", [1, 2, 3, 4, 5])
def test_operators_bit_identical_to_oracle(gpu_lib, N):
    o = po.Oracle(po.make_config(po.SYS_EULER, N, 2, 2))
    for mine, theirs in OPS:
        a, b = aderdg.operator(N, mine), o.operator(theirs)
        assert a.shape == b.shape
        assert np.array_equal(a, b), (N, mine, np.abs(a - b).max())


@pytest.mark.parametrize("name", ["ad_sine", "euler_vortex", "euler_rp2d", "bn_cylinder"])
def test_initial_field_bit_identical_to_oracle(gpu_lib, name):
    cfg, ic, params, _ = aderdg.workloads.make(name, side=9, N=3)
    uh, lh = aderdg.project_initial_condition(cfg, ic, params)
    o = po.Oracle(oracle_config(cfg))
    uo, lo = o.project_ic(ic, params)
    assert np.array_equal(uh, uo)
    assert np.array_equal(lh, lo)


def test_reference_initial_fields(gpu_lib):
    cfg = aderdg.Config(system=aderdg.SYS_EULER, N=1, imax=24, jmax=6, xr=(4.0, 1.0), bc_mode=1)
    uh, lh = aderdg.project_initial_condition(cfg, aderdg.IC_EULER_DMR)
    o = po.Oracle(oracle_config(cfg))
    uo, lo = o.project_ic(po.IC_EULER_DMR, ())
    assert np.array_equal(uh, uo) and np.array_equal(lh, lo)
    for t in (1, 2, 3, 7):
        cfg = aderdg.Config(system=aderdg.SYS_BN, N=2, imax=10, jmax=2, xl=(-0.5, -0.05), xr=(0.5, 0.05))
        uh, lh = aderdg.project_initial_condition(cfg, aderdg.IC_BN_RP1D, (t, 0.0))
        uo, lo = po.Oracle(oracle_config(cfg)).project_ic(po.IC_BN_RP1D, (t, 0.0))
        assert np.array_equal(uh, uo) and np.array_equal(lh, lo)


BAD = [dict(N=0), dict(N=6), dict(imax=0), dict(xr=(0.0, 1.0)), dict(cfl=0.0), dict(precision=7), dict(bc=(2, 1, 1, 1)),
       dict(bc=(0, 1, 1, 1)), dict(system=3), dict(bc_mode=1, system=aderdg.SYS_BN), dict(gamma=1.0)]


@pytest.mark.parametrize("over", BAD)
def test_create_rejects_bad_config(gpu_lib, over):
    cfg = aderdg.Config(**over)
    with pytest.raises(aderdg.AderdgError) as e:
        aderdg.Solver(cfg)
    assert e.value.code in (-1, -7)


def test_null_arguments_are_errors_not_crashes(gpu_lib):
    L = gpu_lib
    assert L.aderdg_create(None, None) == -1
    assert L.aderdg_upload(None, None) == -1
    assert L.aderdg_step(None, None, 1.0, None, None) == -1
    assert L.aderdg_destroy(None) == 0
    assert L.aderdg_operator(0, 0, None) == -1
    out = np.zeros(4)
    assert L.aderdg_operator(3, 99, out.ctypes.data_as(ctypes.POINTER(ctypes.c_double))) == -1


def test_workload_definitions():
    mix = aderdg.workloads.request_mix(256, seed=1)
    assert len(mix) == 256
    assert {m["name"] for m in mix} == set(aderdg.workloads.WORKLOADS)
    assert all(2 <= m["N"] <= 5 and 32 <= m["side"] <= 512 for m in mix)
    cfg, ic, p, tend = aderdg.workloads.make("euler_vortex")
    assert (cfg.N, cfg.imax, cfg.jmax, tend) == (4, 256, 256, 10.0)
    assert cfg.dofs == 4 * 25 * 65536


def test_noalloc_entry_validates_like_create(gpu_lib):
    """The allocation-free time step refuses what aderdg_create refuses (N
    outside 1..5, a bad precision), before it touches the device."""
    f = gpu_lib.aderdg_calc_time_step_noalloc
    f.restype = ctypes.c_int
    f.argtypes = [ctypes.POINTER(aderdg.core._Config), ctypes.c_void_p, ctypes.c_double, ctypes.c_double,
                  ctypes.c_void_p, ctypes.c_void_p]
    dummy = ctypes.c_double(0)
    for over, code in ((dict(N=6), -7), (dict(N=0), -7), (dict(precision=7), -1)):
        cfg = dataclasses.replace(aderdg.Config(system=aderdg.SYS_EULER, N=3, imax=8, jmax=8), **over)
        c = cfg.to_c()
        assert f(ctypes.byref(c), ctypes.addressof(dummy), 0.0, 1.0, ctypes.addressof(dummy), None) == code
        c2 = cfg.to_c()
        h = ctypes.c_void_p()
        assert gpu_lib.aderdg_create(ctypes.byref(c2), ctypes.byref(h)) == code


def test_tuning_table_round_trip(gpu_lib):
    """The tuner's table: set, read back, and refused outside the candidates."""
    n_pred, n_cells = aderdg.tuning_variants()
    assert n_pred >= 2 and n_cells >= 2
    old = aderdg.get_tuning(aderdg.SYS_BN, 4, aderdg.FP32_WIDE)
    aderdg.set_tuning(aderdg.SYS_BN, 4, aderdg.FP32_WIDE, predictor=n_pred - 1, cells=1, subcell_per_sm=2)
    assert aderdg.get_tuning(aderdg.SYS_BN, 4, aderdg.FP32_WIDE) == dict(predictor=n_pred - 1, cells=1,
                                                                        subcell_per_sm=2)
    for bad in (dict(predictor=n_pred), dict(cells=n_cells), dict(predictor=-1), dict(subcell_per_sm=-1)):
        with pytest.raises(aderdg.AderdgError):
            aderdg.set_tuning(aderdg.SYS_BN, 4, aderdg.FP32_WIDE, **bad)
    with pytest.raises(aderdg.AderdgError):
        aderdg.set_tuning(aderdg.SYS_BN, 6, aderdg.FP32_WIDE)
    aderdg.set_tuning(aderdg.SYS_BN, 4, aderdg.FP32_WIDE, **old)


def test_shipped_tuning_table_is_complete_and_valid(gpu_lib):
    """The table aderdg.load applies (aderdg/tuning_gb300.json): one entry per
    (system, N, FP32 mode), every choice among the library's candidates, and
    the library holds exactly those choices after loading."""
    import json
    n_pred, n_cells = aderdg.tuning_variants()
    with open(aderdg.core.TUNING_FILE) as fh:
        table = json.load(fh)
    entries = table["entries"]
    keys = {"%d_%d_%d" % (s, n, p) for s in (0, 1, 2) for n in (1, 2, 3, 4, 5)
            for p in (aderdg.FP32_MIXED, aderdg.FP32_WIDE)}
    assert set(entries) == keys
    for k, e in entries.items():
        assert 0 <= e["predictor"] < n_pred and 0 <= e["cells"] < n_cells and 0 <= e["subcell_per_sm"] <= 3, k
        s, n, p = (int(x) for x in k.split("_"))
        if os.environ.get("ADERDG_TUNING") is None:
            assert aderdg.get_tuning(s, n, p) == {q: e[q] for q in ("predictor", "cells", "subcell_per_sm")}, k
