"""ctypes binding of the CPU oracle (oracle.cpp).

TEST INFRASTRUCTURE ONLY: imported by tests/, by the smoke() check of
__graft_entry__.py and by the cpu_baseline / reference legs of bench.py.  The
product library never uses it.  Parity with the real Fortran reference is
unpinned (no reference tests or golden vectors exist and no Fortran compiler is
available); see oracle.h.
"""
import ctypes
import os
import subprocess

import numpy as np

_HERE = os.path.dirname(os.path.abspath(__file__))
_LIB_PATH = os.path.join(_HERE, "_build", "liboracle.so")

SYS_ADVDIFF, SYS_EULER, SYS_BN = 0, 1, 2
NVAR = {SYS_ADVDIFF: 1, SYS_EULER: 4, SYS_BN: 9}

(UH, OLDUH, DUH, QHI, FHI, SHI, QBND, FBND, GRADQBND, FU, GU, FM, FP, GM, GP, LH, NEWLH,
 LMIN, LMAX, LMIN_OLD, LMAX_OLD) = range(21)
RECOMPUTE, STATUS, OLDSTATUS = range(3)
(OP_XI, OP_W, OP_MM, OP_IMM, OP_KXI, OP_DUDX, OP_F0, OP_K1, OP_IK1, OP_FL, OP_FR, OP_UH2LIM,
 OP_LIM2UH, OP_UH2LOB, OP_XILOB, OP_WLOB, OP_XILIMBARY) = range(17)

IC_AD_ZERO, IC_AD_SINE = 0, 1
IC_EULER_DMR, IC_EULER_VORTEX, IC_EULER_RP2D = 10, 11, 12
IC_BN_RP1D, IC_BN_CYLINDER = 20, 21


class OracleConfig(ctypes.Structure):
    _fields_ = [
        ("system", ctypes.c_int), ("N", ctypes.c_int),
        ("imax", ctypes.c_int), ("jmax", ctypes.c_int),
        ("xl", ctypes.c_double * 2), ("xr", ctypes.c_double * 2),
        ("bc", ctypes.c_int * 4), ("bc_mode", ctypes.c_int),
        ("cfl", ctypes.c_double), ("gamma", ctypes.c_double),
        ("gamma_s", ctypes.c_double), ("gamma_g", ctypes.c_double),
        ("pi_s", ctypes.c_double), ("pi_g", ctypes.c_double),
        ("cx", ctypes.c_double), ("cy", ctypes.c_double), ("a", ctypes.c_double),
        ("ad_flux_mode", ctypes.c_int), ("limiter", ctypes.c_int),
    ]


def build():
    """Compile liboracle.so from oracle.cpp (make in this directory)."""
    subprocess.run(["make", "-s", "-C", _HERE], check=True)
    return _LIB_PATH


_lib = None


def lib():
    global _lib
    if _lib is None:
        if not os.path.exists(_LIB_PATH):
            build()
        L = ctypes.CDLL(_LIB_PATH)
        vp, dp, ip, i, d = ctypes.c_void_p, ctypes.POINTER(ctypes.c_double), ctypes.POINTER(ctypes.c_int), ctypes.c_int, ctypes.c_double
        cfgp = ctypes.POINTER(OracleConfig)
        sig = {
            "oracle_create": (vp, [cfgp]), "oracle_destroy": (None, [vp]),
            "oracle_array_size": (ctypes.c_long, [vp, i]),
            "oracle_set_uh": (i, [vp, dp]), "oracle_get_array": (i, [vp, i, dp]),
            "oracle_set_array": (i, [vp, i, dp]), "oracle_get_int_array": (i, [vp, i, ip]),
            "oracle_set_int_array": (i, [vp, i, ip]), "oracle_get_operator": (i, [vp, i, dp]),
            "oracle_init_limiter": (i, [vp, dp]), "oracle_calc_time_step": (d, [vp, d, d]),
            "oracle_set_dt": (None, [vp, d]), "oracle_set_time": (None, [vp, d]),
            "oracle_get_min_max": (None, [vp]), "oracle_save_olduh": (None, [vp]),
            "oracle_predictor": (None, [vp]), "oracle_volume_integral": (None, [vp]),
            "oracle_riemann": (None, [vp]), "oracle_surface_integral": (None, [vp]),
            "oracle_element_update": (i, [vp]), "oracle_limiter": (None, [vp]),
            "oracle_step": (i, [vp, dp, d, dp]),
            "oracle_initial_field": (i, [cfgp, i, dp, d, d, dp]),
            "oracle_project_ic": (i, [vp, i, dp, dp, dp]),
        }
        for name, (res, args) in sig.items():
            f = getattr(L, name)
            f.restype = res
            f.argtypes = args
        _lib = L
    return _lib


def _dptr(a):
    return a.ctypes.data_as(ctypes.POINTER(ctypes.c_double))


def _iptr(a):
    return a.ctypes.data_as(ctypes.POINTER(ctypes.c_int))


def make_config(system, N, imax, jmax, xl=(0.0, 0.0), xr=(1.0, 1.0), bc=(1, 1, 1, 1), bc_mode=0,
                cfl=0.9, gamma=1.4, gamma_s=1.4, gamma_g=1.4, pi_s=0.0, pi_g=0.0,
                cx=1.0, cy=1.0, a=1e-3, ad_flux_mode=0, limiter=1):
    c = OracleConfig()
    c.system, c.N, c.imax, c.jmax = system, N, imax, jmax
    c.xl[0], c.xl[1] = xl
    c.xr[0], c.xr[1] = xr
    for k in range(4):
        c.bc[k] = bc[k]
    c.bc_mode, c.cfl, c.gamma = bc_mode, cfl, gamma
    c.gamma_s, c.gamma_g, c.pi_s, c.pi_g = gamma_s, gamma_g, pi_s, pi_g
    c.cx, c.cy, c.a = cx, cy, a
    c.ad_flux_mode, c.limiter = ad_flux_mode, limiter
    return c


class Oracle:
    """One oracle instance: the reference's module state for one grid."""

    def __init__(self, cfg):
        self.cfg = cfg
        self.L = lib()
        self.h = self.L.oracle_create(ctypes.byref(cfg))
        if not self.h:
            raise ValueError("oracle_create failed")
        self.V = NVAR[cfg.system]
        self.P = cfg.N + 1
        self.S = 2 * cfg.N + 1

    def __del__(self):
        h = getattr(self, "h", None)
        if h:
            self.L.oracle_destroy(h)
            self.h = None

    def get(self, which):
        n = self.L.oracle_array_size(self.h, which)
        out = np.empty(n, dtype=np.float64)
        assert self.L.oracle_get_array(self.h, which, _dptr(out)) == 0
        return out

    def set(self, which, arr):
        arr = np.ascontiguousarray(arr, dtype=np.float64).ravel()
        assert arr.size == self.L.oracle_array_size(self.h, which)
        assert self.L.oracle_set_array(self.h, which, _dptr(arr)) == 0

    def get_int(self, which):
        out = np.empty(self.cfg.imax * self.cfg.jmax, dtype=np.int32)
        assert self.L.oracle_get_int_array(self.h, which, _iptr(out)) == 0
        return out

    def set_int(self, which, arr):
        arr = np.ascontiguousarray(arr, dtype=np.int32).ravel()
        assert self.L.oracle_set_int_array(self.h, which, _iptr(arr)) == 0

    def operator(self, which):
        out = np.empty(4 * (self.S + 2) ** 2, dtype=np.float64)
        n = self.L.oracle_get_operator(self.h, which, _dptr(out))
        assert n > 0
        return out[:n].copy()

    def project_ic(self, ic, params):
        p = np.zeros(32, dtype=np.float64)
        p[: len(params)] = params
        uh = np.empty(self.L.oracle_array_size(self.h, UH), dtype=np.float64)
        lh = np.empty(self.L.oracle_array_size(self.h, LH), dtype=np.float64)
        assert self.L.oracle_project_ic(self.h, ic, _dptr(p), _dptr(uh), _dptr(lh)) == 0
        return uh, lh

    def init_limiter(self, lh_ic):
        lh_ic = np.ascontiguousarray(lh_ic, dtype=np.float64)
        return self.L.oracle_init_limiter(self.h, _dptr(lh_ic))

    def calc_time_step(self, time, tend):
        return self.L.oracle_calc_time_step(self.h, time, tend)

    def step(self, time, tend):
        t = ctypes.c_double(time)
        dt = ctypes.c_double(0.0)
        nrec = self.L.oracle_step(self.h, ctypes.byref(t), tend, ctypes.byref(dt))
        return t.value, dt.value, nrec

    # individual phases of main.f90's loop body
    def set_dt(self, dt):
        self.L.oracle_set_dt(self.h, dt)

    def set_time(self, t):
        self.L.oracle_set_time(self.h, t)

    def get_min_max(self):
        self.L.oracle_get_min_max(self.h)

    def save_olduh(self):
        self.L.oracle_save_olduh(self.h)

    def predictor(self):
        self.L.oracle_predictor(self.h)

    def volume_integral(self):
        self.L.oracle_volume_integral(self.h)

    def riemann(self):
        self.L.oracle_riemann(self.h)

    def surface_integral(self):
        self.L.oracle_surface_integral(self.h)

    def element_update(self):
        return self.L.oracle_element_update(self.h)

    def limiter(self):
        self.L.oracle_limiter(self.h)


def initial_field(cfg, ic, params, x, y):
    p = np.zeros(32, dtype=np.float64)
    p[: len(params)] = params
    out = np.zeros(9, dtype=np.float64)
    assert lib().oracle_initial_field(ctypes.byref(cfg), ic, _dptr(p), x, y, _dptr(out)) == 0
    return out[: NVAR[cfg.system]]
