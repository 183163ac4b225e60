"""The allocation-free time-step entry point, for callers that cannot call
cudaMalloc (their device memory comes from a host framework's pool or another
runtime, or they must avoid the synchronisation an allocation can cause).

aderdg_calc_time_step_noalloc takes the state and the output as device
pointers owned by the caller -- here torch tensors -- and keeps its scratch
in a fixed device array inside the library.  Its time step must equal the
one of the context API's aderdg_calc_time_step exactly (the tolerance the
parity tests use for dt), on two calls in a row, which also checks that the
shared scratch is left clean between calls.  This file is collected last.
"""
import ctypes

import numpy as np
import pytest

import aderdg

pytestmark = pytest.mark.gpu


def _entry(lib):
    f = lib.aderdg_calc_time_step_noalloc
    f.restype = ctypes.c_int
    f.argtypes = [ctypes.POINTER(aderdg.core._Config), ctypes.c_void_p, ctypes.c_double, ctypes.c_double,
                  ctypes.c_void_p, ctypes.c_void_p]
    return f


@pytest.mark.parametrize("name,N,side", [("euler_vortex", 4, 48), ("euler_rp2d", 3, 40), ("bn_cylinder", 3, 33),
                                         ("ad_sine", 2, 16)])
def test_noalloc_time_step_matches_context_api(gpu_lib, name, N, side):
    torch = pytest.importorskip("torch")
    f = _entry(gpu_lib)
    cfg, ic, params, tend = aderdg.workloads.make(name, side=side, N=N)
    uh, _ = aderdg.project_initial_condition(cfg, ic, params)
    s = aderdg.Solver(cfg)
    s.upload(uh)
    for time in (0.0, 0.5 * tend):
        dt_ref = s.calc_time_step(time, tend)
        uh_dev = torch.from_numpy(uh).to("cuda")
        dt_dev = torch.full((2,), -1.0, dtype=torch.float64, device="cuda")
        stream = torch.cuda.current_stream().cuda_stream
        c = cfg.to_c()
        for k in range(2):  # two calls in a row share the scratch array
            r = f(ctypes.byref(c), uh_dev.data_ptr(), time, tend, dt_dev.data_ptr() + 8 * k, stream)
            assert r == 0, gpu_lib.aderdg_last_error(None)
        torch.cuda.synchronize()
        got = dt_dev.cpu().numpy()
        assert got[0] == dt_ref and got[1] == dt_ref, (got, dt_ref)
    s.close()


def test_noalloc_time_step_after_state_change(gpu_lib):
    """A different state after a first call: the second call sees only its own input."""
    torch = pytest.importorskip("torch")
    f = _entry(gpu_lib)
    cfg, ic, params, tend = aderdg.workloads.make("euler_rp2d", side=24, N=3)
    uh, _ = aderdg.project_initial_condition(cfg, ic, params)
    s = aderdg.Solver(cfg)
    s.upload(uh)
    t, _, _ = s.step(0.0, tend)
    u1, _ = s.download()
    dt_ref0 = aderdg.Solver(cfg)
    dt_ref0.upload(uh)
    ref0 = dt_ref0.calc_time_step(0.0, tend)
    ref1 = s.calc_time_step(t, tend)
    c = cfg.to_c()
    out = torch.zeros(2, dtype=torch.float64, device="cuda")
    stream = torch.cuda.current_stream().cuda_stream
    for k, (u, time) in enumerate(((uh, 0.0), (u1, t))):
        ud = torch.from_numpy(np.ascontiguousarray(u)).to("cuda")
        assert f(ctypes.byref(c), ud.data_ptr(), time, tend, out.data_ptr() + 8 * k, stream) == 0
        torch.cuda.synchronize()
    got = out.cpu().numpy()
    assert got[0] == ref0 and got[1] == ref1


def test_noalloc_rejects_grids_beyond_its_scratch(gpu_lib):
    f = _entry(gpu_lib)
    cfg = aderdg.Config(system=aderdg.SYS_EULER, N=1, imax=2048, jmax=1025)
    c = cfg.to_c()
    dummy = ctypes.c_double(0)
    r = f(ctypes.byref(c), ctypes.addressof(dummy), 0.0, 1.0, ctypes.addressof(dummy), None)
    assert r == -8
    assert b"exceed the maximum" in gpu_lib.aderdg_last_error(None)
