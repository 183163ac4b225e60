"""ctypes binding of libaderdg_gpu.so (include/aderdg_gpu.h).

The Solver class mirrors the reference driver (Euler/main.f90:24-100): one
method per phase of the loop body, plus the fused step and the fused run.
Arrays use the reference's Fortran layouts, flattened in Fortran order.
There is no CPU fallback: every call goes to the CUDA library, and a missing
library or a failing CUDA call raises.
"""
import ctypes
import json
import dataclasses
import os

import numpy as np

from . import builder as _build

SYS_ADVDIFF, SYS_EULER, SYS_BN = 0, 1, 2
NVAR = {SYS_ADVDIFF: 1, SYS_EULER: 4, SYS_BN: 9}
# precision modes (aderdg_precision): FP64 throughout; FP32 contractions with
# the FP64 split of the mixed mode; FP32-wide (faster, FP32 BN faces and subcell
# re-solve, uncertified DMP comparisons)
FP64, FP32_MIXED, FP32_WIDE = 0, 1, 2

(A_UH, A_DUH, A_QHI, A_FHI, A_SHI, A_QBND, A_FBND, A_GRADQBND, A_FU, A_GU, A_FP, A_GP, A_LH, A_LMIN,
 A_LMAX, A_RECOMPUTE, A_STATUS) = range(17)
INT_ARRAYS = (A_RECOMPUTE, A_STATUS)

IC_AD_ZERO, IC_AD_SINE = 0, 1
IC_EULER_DMR, IC_EULER_VORTEX, IC_EULER_RP2D = 10, 11, 12
IC_BN_RP1D, IC_BN_CYLINDER = 20, 21

ERRORS = {0: "OK", -1: "EINVAL", -2: "ENOMEM", -3: "ECUDA", -4: "ETIMEOUT", -5: "ENONFINITE", -6: "ESTATE",
          -7: "EUNSUPPORTED", -8: "ENOSPACE"}


class AderdgError(RuntimeError):
    def __init__(self, code, msg):
        super().__init__("%s (%d): %s" % (ERRORS.get(code, "?"), code, msg))
        self.code = code


class _Config(ctypes.Structure):
    _fields_ = [
        ("system", ctypes.c_int), ("N", ctypes.c_int), ("imax", ctypes.c_int), ("jmax", ctypes.c_int),
        ("xl", ctypes.c_double * 2), ("xr", ctypes.c_double * 2), ("bc", ctypes.c_int * 4),
        ("bc_mode", ctypes.c_int), ("cfl", ctypes.c_double), ("gamma", ctypes.c_double),
        ("gamma_s", ctypes.c_double), ("gamma_g", ctypes.c_double), ("pi_s", ctypes.c_double),
        ("pi_g", ctypes.c_double), ("cx", ctypes.c_double), ("cy", ctypes.c_double), ("a", ctypes.c_double),
        ("ad_flux_mode", ctypes.c_int), ("limiter", ctypes.c_int), ("precision", ctypes.c_int),
    ]


class _Info(ctypes.Structure):
    _fields_ = [("cells", ctypes.c_long), ("dofs", ctypes.c_long), ("device_bytes", ctypes.c_long),
                ("steps", ctypes.c_long), ("time", ctypes.c_double), ("dt", ctypes.c_double),
                ("n_recompute", ctypes.c_int), ("n_limited", ctypes.c_int), ("n_settled", ctypes.c_int),
                ("n_listed", ctypes.c_int)]


class _Tuning(ctypes.Structure):
    _fields_ = [("predictor", ctypes.c_int), ("cells", ctypes.c_int), ("subcell_per_sm", ctypes.c_int)]


@dataclasses.dataclass
class Config:
    """What the reference reads from params.ini plus its compile-time N and CFL."""
    system: int = SYS_EULER
    N: int = 3
    imax: int = 16
    jmax: int = 16
    xl: tuple = (0.0, 0.0)
    xr: tuple = (1.0, 1.0)
    bc: tuple = (1, 1, 1, 1)
    bc_mode: int = 0
    cfl: float = 0.9
    gamma: float = 1.4
    gamma_s: float = 1.4
    gamma_g: float = 1.4
    pi_s: float = 0.0
    pi_g: float = 0.0
    cx: float = 1.0
    cy: float = 1.0
    a: float = 1e-3
    ad_flux_mode: int = 0
    limiter: int = 1
    precision: int = FP64

    @property
    def nvar(self):
        return NVAR[self.system]

    @property
    def P(self):
        return self.N + 1

    @property
    def S(self):
        return 2 * self.N + 1

    @property
    def cells(self):
        return self.imax * self.jmax

    @property
    def dofs(self):
        """DOF-updates per step: nVar (N+1)^2 per cell."""
        return self.nvar * self.P * self.P * self.cells

    def to_c(self):
        c = _Config()
        c.system, c.N, c.imax, c.jmax = self.system, self.N, self.imax, self.jmax
        c.xl[0], c.xl[1] = self.xl
        c.xr[0], c.xr[1] = self.xr
        for k in range(4):
            c.bc[k] = self.bc[k]
        c.bc_mode, c.cfl, c.gamma = self.bc_mode, self.cfl, self.gamma
        c.gamma_s, c.gamma_g, c.pi_s, c.pi_g = self.gamma_s, self.gamma_g, self.pi_s, self.pi_g
        c.cx, c.cy, c.a = self.cx, self.cy, self.a
        c.ad_flux_mode, c.limiter, c.precision = self.ad_flux_mode, self.limiter, self.precision
        return c


_lib = None


def library_path():
    return _build.LIB_PATH


def load(build_if_missing=False):
    """Load libaderdg_gpu.so; raises when it is not built (no fallback)."""
    global _lib
    if _lib is not None:
        return _lib
    path = library_path()
    if not os.path.exists(path):
        if not build_if_missing:
            raise RuntimeError("libaderdg_gpu.so is not built (%s); run aderdg.build.build()" % path)
        _build.build()
    L = ctypes.CDLL(path)
    vp, dp, ip, i, d = ctypes.c_void_p, ctypes.POINTER(ctypes.c_double), ctypes.POINTER(ctypes.c_int), ctypes.c_int, ctypes.c_double
    cfgp = ctypes.POINTER(_Config)
    sig = {
        "aderdg_create": (i, [cfgp, ctypes.POINTER(vp)]), "aderdg_destroy": (i, [vp]),
        "aderdg_upload": (i, [vp, dp]), "aderdg_init_limiter": (i, [vp, dp, ip]),
        "aderdg_upload_limiter": (i, [vp, ip, dp]), "aderdg_download_limiter": (i, [vp, ip, dp]),
        "aderdg_download": (i, [vp, dp, ip]),
        "aderdg_calc_time_step": (i, [vp, d, d, dp]), "aderdg_set_time_step": (i, [vp, d, d]),
        "aderdg_limiter_prepare": (i, [vp]), "aderdg_space_time_predictor": (i, [vp]),
        "aderdg_volume_integral": (i, [vp]), "aderdg_riemann_problem": (i, [vp]),
        "aderdg_surface_integral": (i, [vp]), "aderdg_element_update": (i, [vp, ip]),
        "aderdg_limiter": (i, [vp]), "aderdg_step": (i, [vp, dp, d, dp, ip]),
        "aderdg_run": (i, [vp, dp, d, i, i, ip]), "aderdg_array_size": (ctypes.c_long, [vp, i]),
        "aderdg_get_array": (i, [vp, i, vp]), "aderdg_get_info": (i, [vp, ctypes.POINTER(_Info)]),
        "aderdg_last_error": (ctypes.c_char_p, [vp]),
        "aderdg_project_initial_condition": (i, [cfgp, i, dp, dp, dp]),
        "aderdg_probe_peaks": (i, [dp, dp]), "aderdg_probe_math": (i, [i, dp, dp]),
        "aderdg_set_array": (i, [vp, i, vp]),
        "aderdg_host_alloc": (i, [ctypes.c_size_t, ctypes.POINTER(vp)]), "aderdg_host_free": (i, [vp]),
        "aderdg_operator": (i, [i, i, dp]), "aderdg_step_host": (i, [vp, dp, dp, d, dp, ip]),
        "aderdg_time_steps": (i, [vp, dp, d, i, i, dp]), "aderdg_profile_step": (i, [vp, dp, d, dp]),
        "aderdg_batch_unit_bytes": (ctypes.c_long, [i, i, i, i]),
        "aderdg_batch_create": (i, [i, i, i, i, ctypes.c_long, i, ctypes.POINTER(vp)]),
        "aderdg_batch_destroy": (i, [vp]),
        "aderdg_batch_admit": (i, [vp, cfgp, dp, dp, d, ctypes.c_long, ip]),
        "aderdg_batch_release": (i, [vp, i]), "aderdg_batch_launch": (i, [vp, i]), "aderdg_batch_sync": (i, [vp, ip]),
        "aderdg_batch_ready": (i, [vp, ip]),
        "aderdg_batch_query": (i, [vp, i, dp, dp, ctypes.POINTER(ctypes.c_long), ip]),
        "aderdg_batch_download": (i, [vp, i, dp]), "aderdg_batch_download_status": (i, [vp, i, ip]),
        "aderdg_batch_counters": (i, [vp, ip, ip, ip]),
        "aderdg_batch_info": (i, [vp, ctypes.POINTER(ctypes.c_long), ctypes.POINTER(ctypes.c_long),
                                  ctypes.POINTER(ctypes.c_long), ip]),
        "aderdg_batch_last_error": (ctypes.c_char_p, [vp]), "aderdg_batch_profile": (i, [vp, dp]),
        "aderdg_batch_run_timed": (i, [ctypes.POINTER(vp), i, i, dp]),
        "aderdg_initial_condition": (i, [vp, i, dp, ip]),
        "aderdg_batch_admit_ic": (i, [vp, cfgp, i, dp, d, ctypes.c_long, ip]),
        "aderdg_cell_averages": (i, [vp, i, dp]), "aderdg_batch_cell_averages": (i, [vp, i, i, dp]),
        "aderdg_error_norms": (i, [vp, i, dp, i, dp]),
        "aderdg_set_tuning": (i, [i, i, i, ctypes.POINTER(_Tuning)]),
        "aderdg_get_tuning": (i, [i, i, i, ctypes.POINTER(_Tuning)]),
        "aderdg_tuning_variants": (i, [ip, ip]),
    }
    for name, (res, args) in sig.items():
        f = getattr(L, name)
        f.restype = res
        f.argtypes = args
    _lib = L
    tuning_file = os.environ.get("ADERDG_TUNING", TUNING_FILE)
    if tuning_file and os.path.exists(tuning_file):
        apply_tuning(load_tuning(tuning_file))
    return L


# The tuner's table measured on the GB300 (aderdg/tuner.py), applied when the
# library is loaded; ADERDG_TUNING names another file ("" for none).
TUNING_FILE = os.path.join(os.path.dirname(os.path.abspath(__file__)), "tuning_gb300.json")
PRECISION_NAMES = {0: "fp64", 1: "fp32_mixed", 2: "fp32_wide"}


def set_tuning(system, N, precision, predictor=0, cells=0, subcell_per_sm=0):
    t = _Tuning(predictor, cells, subcell_per_sm)
    r = load().aderdg_set_tuning(system, N, precision, ctypes.byref(t))
    if r:
        raise AderdgError(r, "bad tuning entry")


def get_tuning(system, N, precision):
    t = _Tuning()
    r = load().aderdg_get_tuning(system, N, precision, ctypes.byref(t))
    if r:
        raise AderdgError(r, "bad tuning key")
    return dict(predictor=t.predictor, cells=t.cells, subcell_per_sm=t.subcell_per_sm)


def tuning_variants():
    a, b = ctypes.c_int(0), ctypes.c_int(0)
    load().aderdg_tuning_variants(ctypes.byref(a), ctypes.byref(b))
    return a.value, b.value


def load_tuning(path):
    with open(path) as fh:
        return json.load(fh)


def apply_tuning(table):
    """Sets every entry of a tuner table {"entries": {"<system>_<N>_<precision>": {...}}}."""
    for key, e in table.get("entries", {}).items():
        system, N, prec = (int(x) for x in key.split("_"))
        t = _Tuning(int(e.get("predictor", 0)), int(e.get("cells", 0)), int(e.get("subcell_per_sm", 0)))
        _lib.aderdg_set_tuning(system, N, prec, ctypes.byref(t))


EXPORTED = ("aderdg_create", "aderdg_destroy", "aderdg_upload", "aderdg_init_limiter", "aderdg_upload_limiter",
            "aderdg_download_limiter", "aderdg_download", "aderdg_calc_time_step", "aderdg_set_time_step",
            "aderdg_limiter_prepare", "aderdg_space_time_predictor", "aderdg_volume_integral",
            "aderdg_riemann_problem", "aderdg_surface_integral", "aderdg_element_update", "aderdg_limiter",
            "aderdg_step", "aderdg_run", "aderdg_array_size", "aderdg_get_array", "aderdg_get_info",
            "aderdg_last_error", "aderdg_project_initial_condition", "aderdg_probe_peaks", "aderdg_set_array",
            "aderdg_operator", "aderdg_step_host", "aderdg_time_steps", "aderdg_profile_step",
            "aderdg_batch_unit_bytes", "aderdg_batch_create", "aderdg_batch_destroy", "aderdg_batch_admit",
            "aderdg_batch_release", "aderdg_batch_launch", "aderdg_batch_sync", "aderdg_batch_ready", "aderdg_batch_query",
            "aderdg_batch_download", "aderdg_batch_download_status", "aderdg_batch_counters", "aderdg_batch_info", "aderdg_batch_last_error", "aderdg_batch_profile",
            "aderdg_batch_run_timed", "aderdg_initial_condition", "aderdg_batch_admit_ic",
            "aderdg_cell_averages", "aderdg_batch_cell_averages", "aderdg_error_norms", "aderdg_host_alloc",
            "aderdg_host_free", "aderdg_set_tuning", "aderdg_get_tuning", "aderdg_tuning_variants",
            "aderdg_probe_math")


def _dp(a):
    return a.ctypes.data_as(ctypes.POINTER(ctypes.c_double))


def _ip(a):
    return a.ctypes.data_as(ctypes.POINTER(ctypes.c_int))


def project_initial_condition(cfg, ic, params=()):
    """Initial field at the Gauss-Legendre nodes (uh) and subcell barycentres (lh_ic)."""
    L = load()
    p = np.zeros(32, dtype=np.float64)
    p[: len(params)] = params
    uh = np.empty(cfg.dofs, dtype=np.float64)
    lh = np.empty(cfg.nvar * cfg.S * cfg.S * cfg.cells, dtype=np.float64)
    c = cfg.to_c()
    r = L.aderdg_project_initial_condition(ctypes.byref(c), ic, _dp(p), _dp(uh), _dp(lh))
    if r:
        raise AderdgError(r, L.aderdg_last_error(None).decode())
    return uh, lh


(OP_XI, OP_W, OP_KXI, OP_DUDX, OP_IK1, OP_F0, OP_FL, OP_FR, OP_UH2LIM, OP_LIM2UH, OP_UH2LOB,
 OP_XILIMBARY) = range(12)


def operator(N, which):
    """Host-built 1D operator of degree N (column-major, flattened)."""
    L = load()
    out = np.zeros(256, dtype=np.float64)
    n = L.aderdg_operator(N, which, _dp(out))
    if n < 0:
        raise AderdgError(n, "bad operator request")
    return out[:n].copy()


class PinnedArray:
    """A float64 numpy array in page-locked host memory (aderdg_host_alloc),
    freed when this object goes away; `.array` is the numpy view."""

    def __init__(self, n):
        L = load()
        self._L = L
        self._p = ctypes.c_void_p()
        r = L.aderdg_host_alloc(ctypes.c_size_t(max(int(n), 1) * 8), ctypes.byref(self._p))
        if r != 0:
            raise AderdgError(r, "aderdg_host_alloc of %d doubles failed" % n)
        buf = (ctypes.c_double * max(int(n), 1)).from_address(self._p.value)
        self.array = np.frombuffer(buf, dtype=np.float64, count=int(n))

    def __del__(self):
        p = getattr(self, "_p", None)
        if p is not None and p.value:
            self._L.aderdg_host_free(p)
            self._p = None


def probe_peaks():
    """(FP64, FP32) FMA throughput of the current device in GFLOP/s."""
    L = load()
    a, b = ctypes.c_double(0), ctypes.c_double(0)
    r = L.aderdg_probe_peaks(ctypes.byref(a), ctypes.byref(b))
    if r:
        raise AderdgError(r, "probe failed")
    return a.value, b.value


def probe_math(x):
    """The FP32-mixed mode's FP64 reciprocal and square root on the device
    beside the correctly rounded ones: array [n, 4] = (rcp, 1/x, sqrt, sqrt(x))."""
    L = load()
    x = np.ascontiguousarray(x, dtype=np.float64)
    out = np.empty((x.size, 4), dtype=np.float64)
    r = L.aderdg_probe_math(int(x.size), _dp(x), _dp(out))
    if r:
        raise AderdgError(r, "probe failed")
    return out


class Solver:
    """One simulation on the GPU: the reference's module state plus its phases."""

    def __init__(self, cfg):
        self.cfg = cfg
        self.L = load()
        self._c = cfg.to_c()
        h = ctypes.c_void_p()
        r = self.L.aderdg_create(ctypes.byref(self._c), ctypes.byref(h))
        if r:
            raise AderdgError(r, self.L.aderdg_last_error(None).decode())
        self.h = h

    def _ck(self, r):
        if r:
            raise AderdgError(r, self.L.aderdg_last_error(self.h).decode())
        return r

    def close(self):
        if getattr(self, "h", None):
            self.L.aderdg_destroy(self.h)
            self.h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def __enter__(self):
        return self

    def __exit__(self, *exc):
        self.close()

    # state transfer
    def upload(self, uh):
        uh = np.ascontiguousarray(uh, dtype=np.float64).ravel()
        assert uh.size == self.cfg.dofs
        self._ck(self.L.aderdg_upload(self.h, _dp(uh)))

    def init_limiter(self, lh_ic):
        n = ctypes.c_int(0)
        lh = None if lh_ic is None else np.ascontiguousarray(lh_ic, dtype=np.float64).ravel()
        self._ck(self.L.aderdg_init_limiter(self.h, None if lh is None else _dp(lh), ctypes.byref(n)))
        return n.value

    def initial_condition(self, ic, params=()):
        """Initial field and initial limiter evaluated on the device; returns
        the number of cells the initial limiter marked."""
        p = np.zeros(32, dtype=np.float64)
        p[: len(params)] = params
        n = ctypes.c_int(0)
        self._ck(self.L.aderdg_initial_condition(self.h, ic, _dp(p), ctypes.byref(n)))
        return n.value

    def cell_averages(self, primitive=True):
        """Cell averages [cell][nVar] of uh (primitive variables by default),
        the field the reference writes to its VTK files."""
        out = np.empty(self.cfg.cells * self.cfg.nvar, dtype=np.float64)
        self._ck(self.L.aderdg_cell_averages(self.h, 1 if primitive else 0, _dp(out)))
        return out.reshape(self.cfg.cells, self.cfg.nvar)

    def error_norms(self, ic, params=(), var=0):
        """(mean |e|, rms e, max |e|) of the cell averages of variable `var`
        against the exact field at the current time."""
        p = np.zeros(32, dtype=np.float64)
        p[: len(params)] = params
        out = np.zeros(3, dtype=np.float64)
        self._ck(self.L.aderdg_error_norms(self.h, ic, _dp(p), var, _dp(out)))
        return tuple(out)

    def upload_limiter(self, status, lh):
        st = np.ascontiguousarray(status, dtype=np.int32).ravel()
        lh = np.ascontiguousarray(lh, dtype=np.float64).ravel()
        self._ck(self.L.aderdg_upload_limiter(self.h, _ip(st), _dp(lh)))

    def download_limiter(self):
        """(status per cell, Lh(nVar, 2N+1, 2N+1, IMAX, JMAX)) of the current state."""
        st = np.empty(self.cfg.cells, dtype=np.int32)
        lh = np.empty(self.cfg.cells * self.cfg.S * self.cfg.S * self.cfg.nvar, dtype=np.float64)
        self._ck(self.L.aderdg_download_limiter(self.h, _ip(st), _dp(lh)))
        return st, lh

    def download(self):
        uh = np.empty(self.cfg.dofs, dtype=np.float64)
        st = np.empty(self.cfg.cells, dtype=np.int32)
        self._ck(self.L.aderdg_download(self.h, _dp(uh), _ip(st)))
        return uh, st

    def download_into(self, uh):
        self._ck(self.L.aderdg_download(self.h, _dp(uh), None))

    # phases of main.f90's loop body
    def calc_time_step(self, time, tend):
        dt = ctypes.c_double(0)
        self._ck(self.L.aderdg_calc_time_step(self.h, time, tend, ctypes.byref(dt)))
        return dt.value

    def set_time_step(self, time, dt):
        self._ck(self.L.aderdg_set_time_step(self.h, time, dt))

    def limiter_prepare(self):
        self._ck(self.L.aderdg_limiter_prepare(self.h))

    def space_time_predictor(self):
        self._ck(self.L.aderdg_space_time_predictor(self.h))

    def volume_integral(self):
        self._ck(self.L.aderdg_volume_integral(self.h))

    def riemann_problem(self):
        self._ck(self.L.aderdg_riemann_problem(self.h))

    def surface_integral(self):
        self._ck(self.L.aderdg_surface_integral(self.h))

    def element_update(self):
        n = ctypes.c_int(0)
        self._ck(self.L.aderdg_element_update(self.h, ctypes.byref(n)))
        return n.value

    def limiter(self):
        self._ck(self.L.aderdg_limiter(self.h))

    # fused
    def step(self, time, tend):
        t = ctypes.c_double(time)
        dt = ctypes.c_double(0)
        n = ctypes.c_int(0)
        self._ck(self.L.aderdg_step(self.h, ctypes.byref(t), tend, ctypes.byref(dt), ctypes.byref(n)))
        return t.value, dt.value, n.value

    def run(self, time, tend, max_steps, sync_every=0):
        t = ctypes.c_double(time)
        n = ctypes.c_int(0)
        self._ck(self.L.aderdg_run(self.h, ctypes.byref(t), tend, max_steps, sync_every, ctypes.byref(n)))
        return t.value, n.value

    def step_host(self, uh, time, tend):
        """One step with host arrays: uh is updated in place (float64, C-contiguous)."""
        assert uh.dtype == np.float64 and uh.flags.c_contiguous and uh.size == self.cfg.dofs
        t = ctypes.c_double(time)
        dt = ctypes.c_double(0)
        n = ctypes.c_int(0)
        self._ck(self.L.aderdg_step_host(self.h, _dp(uh), ctypes.byref(t), tend, ctypes.byref(dt), ctypes.byref(n)))
        return t.value, dt.value, n.value

    # measurement
    def time_steps(self, time, tend, steps, flush_l2=True):
        """Device milliseconds of each of `steps` fused steps."""
        t = ctypes.c_double(time)
        ms = np.zeros(steps, dtype=np.float64)
        self._ck(self.L.aderdg_time_steps(self.h, ctypes.byref(t), tend, steps, 1 if flush_l2 else 0, _dp(ms)))
        return t.value, ms

    PHASES = ("begin", "predictor", "faces", "cells", "mark", "subcell", "end")

    def profile_step(self, time, tend):
        """Device milliseconds of each launch of one fused step."""
        t = ctypes.c_double(time)
        ms = np.zeros(7, dtype=np.float64)
        self._ck(self.L.aderdg_profile_step(self.h, ctypes.byref(t), tend, _dp(ms)))
        return t.value, dict(zip(self.PHASES, ms))

    # introspection
    def get(self, which):
        n = self.L.aderdg_array_size(self.h, which)
        if n < 0:
            raise AderdgError(int(n), "array not available")
        out = np.empty(n, dtype=np.int32 if which in INT_ARRAYS else np.float64)
        self._ck(self.L.aderdg_get_array(self.h, which, out.ctypes.data_as(ctypes.c_void_p)))
        return out

    def set(self, which, arr):
        arr = np.ascontiguousarray(arr, dtype=np.int32 if which in INT_ARRAYS else np.float64).ravel()
        n = self.L.aderdg_array_size(self.h, which)
        assert arr.size == n, (arr.size, n)
        self._ck(self.L.aderdg_set_array(self.h, which, arr.ctypes.data_as(ctypes.c_void_p)))

    def info(self):
        i = _Info()
        self._ck(self.L.aderdg_get_info(self.h, ctypes.byref(i)))
        return {k: getattr(i, k) for k, _ in _Info._fields_}


class Batch:
    """Many independent simulations of one (system, N, precision, limiter) on
    the GPU, stepped together; admit and release them between steps."""

    def __init__(self, system, N, precision=FP64, limiter=1, capacity_units=1 << 16, max_instances=256):
        self.L = load()
        self.system, self.N, self.precision = system, N, precision
        self.limiter = 1 if (limiter and system != SYS_ADVDIFF) else 0
        self.capacity_units = int(capacity_units)
        h = ctypes.c_void_p()
        r = self.L.aderdg_batch_create(system, N, precision, self.limiter, self.capacity_units, max_instances,
                                       ctypes.byref(h))
        if r:
            raise AderdgError(r, self.L.aderdg_last_error(None).decode())
        self.h = h
        self.cfgs = {}

    @staticmethod
    def units(cfg):
        return (cfg.imax + 1) * (cfg.jmax + 1)

    @staticmethod
    def unit_bytes(system, N, precision=FP64, limiter=1):
        return int(load().aderdg_batch_unit_bytes(system, N, precision, limiter))

    def _ck(self, r):
        if r:
            raise AderdgError(r, self.L.aderdg_batch_last_error(self.h).decode())
        return r

    def close(self):
        if getattr(self, "h", None):
            self.L.aderdg_batch_destroy(self.h)
            self.h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def admit(self, cfg, uh, lh_ic=None, tend=1e30, max_steps=0):
        """Returns the slot id, or None when the batch has no room."""
        c = cfg.to_c()
        uh = np.ascontiguousarray(uh, dtype=np.float64).ravel()
        lh = None if lh_ic is None else np.ascontiguousarray(lh_ic, dtype=np.float64).ravel()
        slot = ctypes.c_int(-1)
        r = self.L.aderdg_batch_admit(self.h, ctypes.byref(c), _dp(uh), None if lh is None else _dp(lh), tend,
                                      int(max_steps), ctypes.byref(slot))
        if r == -8:
            return None
        self._ck(r)
        self.cfgs[slot.value] = cfg
        return slot.value

    def admit_ic(self, cfg, ic, params=(), tend=1e30, max_steps=0):
        """Admission with the initial field evaluated on the device; the slot
        id, or None when the batch has no room."""
        c = cfg.to_c()
        p = np.zeros(32, dtype=np.float64)
        p[: len(params)] = params
        slot = ctypes.c_int(-1)
        r = self.L.aderdg_batch_admit_ic(self.h, ctypes.byref(c), ic, _dp(p), tend, int(max_steps), ctypes.byref(slot))
        if r == -8:
            return None
        self._ck(r)
        self.cfgs[slot.value] = cfg
        return slot.value

    def release(self, slot):
        self._ck(self.L.aderdg_batch_release(self.h, slot))
        self.cfgs.pop(slot, None)

    def launch(self, steps):
        self._ck(self.L.aderdg_batch_launch(self.h, steps))

    def sync(self):
        n = ctypes.c_int(0)
        self._ck(self.L.aderdg_batch_sync(self.h, ctypes.byref(n)))
        return n.value

    def ready(self):
        """True when the batch's queued work has completed (sync would not wait)."""
        r = ctypes.c_int(0)
        self._ck(self.L.aderdg_batch_ready(self.h, ctypes.byref(r)))
        return bool(r.value)

    def query(self, slot):
        t, dt, st, done = ctypes.c_double(0), ctypes.c_double(0), ctypes.c_long(0), ctypes.c_int(0)
        r = self.L.aderdg_batch_query(self.h, slot, ctypes.byref(t), ctypes.byref(dt), ctypes.byref(st),
                                      ctypes.byref(done))
        return dict(time=t.value, dt=dt.value, steps=st.value, done=bool(done.value), status=r)

    def download(self, slot, out=None):
        """The simulation's uh; into `out` (a float64 C-contiguous array of at
        least its DOFs, e.g. a PinnedArray's) when given, as a view of it."""
        cfg = self.cfgs[slot]
        if out is None:
            uh = np.empty(cfg.dofs, dtype=np.float64)
        else:
            assert out.dtype == np.float64 and out.flags.c_contiguous and out.size >= cfg.dofs
            uh = out[: cfg.dofs]
        self._ck(self.L.aderdg_batch_download(self.h, slot, _dp(uh)))
        return uh

    def counters(self):
        """The last step's troubled, re-solved and FP64-settled cells, summed over the simulations."""
        a, b, c = ctypes.c_int(0), ctypes.c_int(0), ctypes.c_int(0)
        self._ck(self.L.aderdg_batch_counters(self.h, ctypes.byref(a), ctypes.byref(b), ctypes.byref(c)))
        return dict(n_recompute=a.value, n_listed=b.value, n_settled=c.value)

    def download_status(self, slot):
        """The simulation's limiter status per cell (1: limited by its last step)."""
        st = np.empty(self.cfgs[slot].cells, dtype=np.int32)
        self._ck(self.L.aderdg_batch_download_status(self.h, slot, _ip(st)))
        return st

    def cell_averages(self, slot, primitive=True):
        cfg = self.cfgs[slot]
        out = np.empty(cfg.cells * cfg.nvar, dtype=np.float64)
        self._ck(self.L.aderdg_batch_cell_averages(self.h, slot, 1 if primitive else 0, _dp(out)))
        return out.reshape(cfg.cells, cfg.nvar)

    def profile(self):
        """Device milliseconds of each launch of one eager step of the batch."""
        ms = np.zeros(7, dtype=np.float64)
        self._ck(self.L.aderdg_batch_profile(self.h, _dp(ms)))
        return dict(zip(Solver.PHASES, ms))

    @staticmethod
    def run_timed(batches, steps):
        """Device milliseconds of `steps` steps of all `batches` run concurrently
        (CUDA events bracketing every batch's stream)."""
        L = load()
        arr = (ctypes.c_void_p * len(batches))(*[b.h for b in batches])
        ms = ctypes.c_double(0)
        r = L.aderdg_batch_run_timed(arr, len(batches), int(steps), ctypes.byref(ms))
        if r:
            raise AderdgError(r, L.aderdg_last_error(None).decode())
        return ms.value

    def info(self):
        u, c, b = ctypes.c_long(0), ctypes.c_long(0), ctypes.c_long(0)
        n = ctypes.c_int(0)
        self._ck(self.L.aderdg_batch_info(self.h, ctypes.byref(u), ctypes.byref(c), ctypes.byref(b), ctypes.byref(n)))
        return dict(used_units=u.value, capacity_units=c.value, device_bytes=b.value, instances=n.value)
