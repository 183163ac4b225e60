"""GB300-native ADER-DG time step: host-side interface.

The product is libaderdg_gpu.so (C ABI in include/aderdg_gpu.h); this package
builds it (builder.py), binds it (core.py), defines the named workloads and
the seeded request mix (workloads.py), serves request streams (serving.py),
tunes the FP32 kernel shapes (tuner.py) and writes the reference's output
files (output.py).  The reference's params.ini
files are read by the C++ driver (host/aderdg_driver.cpp).
"""
from .builder import build, LIB_PATH  # noqa: F401
from .core import (  # noqa: F401
    A_DUH, A_FBND, A_FHI, A_FP, A_FU, A_GP, A_GRADQBND, A_GU, A_LH, A_LMAX, A_LMIN, A_QBND, A_QHI, A_RECOMPUTE,
    A_SHI, A_STATUS, A_UH, EXPORTED, FP32_MIXED, FP32_WIDE, FP64, IC_AD_SINE, IC_AD_ZERO, IC_BN_CYLINDER, IC_BN_RP1D,
    IC_EULER_DMR, IC_EULER_RP2D, IC_EULER_VORTEX, NVAR, SYS_ADVDIFF, SYS_BN, SYS_EULER, AderdgError, Config,
    Batch, PinnedArray, Solver, apply_tuning, get_tuning, load, load_tuning, operator, probe_peaks,
    project_initial_condition, set_tuning, tuning_variants)
from .core import (OP_DUDX, OP_F0, OP_FL, OP_FR, OP_IK1, OP_KXI, OP_LIM2UH, OP_UH2LIM, OP_UH2LOB, OP_W,  # noqa: F401
                   OP_XI, OP_XILIMBARY)
from . import workloads  # noqa: F401,E402
from . import serving  # noqa: F401,E402
from . import output  # noqa: F401,E402
