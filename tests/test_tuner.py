"""The autotuner's kernel shapes (aderdg/tuner.py, include/aderdg_gpu.h
aderdg_tuning): every candidate runs and gives the default shape's results --
bit for bit for the cell-kernel and subcell shapes (FP64 reference-order
translation units), to FP32 rounding for the predictor shapes (relative L1 <=
1e-6: each predictor instantiation is compiled with fused multiply-adds, and
the compiler may group the products of one expression differently in each;
measured 4e-7 at most, on the smooth vortex, none on piecewise-constant
fields) -- and the tuner picks a valid shape and leaves it set."""
import numpy as np
import pytest

import aderdg
from helpers import rel_l1

pytestmark = pytest.mark.gpu


@pytest.fixture
def default_tuning(gpu_lib):
    saved = {}
    for s in (0, 1, 2):
        for n in (1, 2, 3, 4, 5):
            for p in (1, 2):
                saved[(s, n, p)] = aderdg.get_tuning(s, n, p)
                aderdg.set_tuning(s, n, p)
    yield
    for (s, n, p), t in saved.items():
        aderdg.set_tuning(s, n, p, **t)


def _run(name, N, side, precision, steps=3):
    cfg, ic, params, tend = aderdg.workloads.make(name, side=side, N=N, precision=precision)
    s = aderdg.Solver(cfg)
    s.initial_condition(ic, params)
    t = 0.0
    for _ in range(steps):
        t, _, _ = s.step(t, tend)
    u, st = s.download()
    s.close()
    return u, st, t


CASES = [("euler_vortex", 4, 16), ("bn_cylinder", 3, 16), ("euler_rp2d", 3, 24), ("ad_sine", 3, 16),
         ("bn_cylinder", 5, 10)]


@pytest.mark.parametrize("precision", [aderdg.FP32_MIXED, aderdg.FP32_WIDE])
@pytest.mark.parametrize("name,N,side", CASES)
def test_every_shape_gives_the_default_results(default_tuning, name, N, side, precision):
    system = aderdg.workloads.WORKLOADS[name]["system"]
    ref, st_ref, t_ref = _run(name, N, side, precision)
    n_pred, n_cells = aderdg.tuning_variants()
    shapes = [dict(predictor=v) for v in range(1, n_pred)] + [dict(cells=v) for v in range(1, n_cells)]
    shapes += [dict(subcell_per_sm=k) for k in (1, 2)]
    for shape in shapes:
        aderdg.set_tuning(system, N, precision, **shape)
        u, st, t = _run(name, N, side, precision)
        aderdg.set_tuning(system, N, precision)
        assert t == t_ref, shape
        if "predictor" in shape:
            assert rel_l1(u, ref) <= 1e-6, (shape, rel_l1(u, ref))
            assert (st != st_ref).sum() == 0, shape
        else:
            assert np.array_equal(u, ref) and np.array_equal(st, st_ref), shape


def test_tuner_picks_a_valid_shape(default_tuning):
    from aderdg import tuner
    r = tuner.tune_one(aderdg.SYS_EULER, 3, aderdg.FP32_MIXED, reps=2, side=48, warm_steps=3)
    n_pred, n_cells = aderdg.tuning_variants()
    assert 0 <= r["predictor"] < n_pred and 0 <= r["cells"] < n_cells and 0 <= r["subcell_per_sm"] <= 3
    assert set(r["ms"]["predictor"]) == set(range(n_pred))
    assert all(v > 0 for v in r["ms"]["predictor"].values())
    got = aderdg.get_tuning(aderdg.SYS_EULER, 3, aderdg.FP32_MIXED)
    assert got == {k: r[k] for k in ("predictor", "cells", "subcell_per_sm")}
