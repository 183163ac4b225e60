"""Builds libaderdg_gpu.so in-tree for sm_103a.

Each (system, N) pair is compiled from two translation units: predictor_tu.cu
(fused multiply-adds) and exact_tu.cu (--fmad=false, reference operation
order), plus the tuner's candidates (predictor_var_tu.cu per variant,
cells_var_tu.cu).  All units compile in parallel; a content hash of the sources and
flags skips the build when nothing changed.
"""
import concurrent.futures
import hashlib
import os
import shutil
import subprocess

PKG_ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))  # .../ader-dg_gb300
CSRC = os.path.join(PKG_ROOT, "csrc")
REPO_ROOT = os.path.dirname(PKG_ROOT)
INCLUDE = os.path.join(REPO_ROOT, "include")
BUILD_DIR = os.path.join(PKG_ROOT, "_build")
LIB_NAME = "libaderdg_gpu.so"
LIB_PATH = os.path.join(BUILD_DIR, LIB_NAME)
DRIVER_PATH = os.path.join(BUILD_DIR, "aderdg_driver")

ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]
SYSTEMS = (0, 1, 2)
DEGREES = (1, 2, 3, 4, 5)
PRED_VARIANTS = 7  # predictor.cuh kPredVariants


def _nvcc():
    cuda = os.environ.get("CUDA_HOME", "/usr/local/cuda")
    p = os.path.join(cuda, "bin", "nvcc")
    return p if os.path.exists(p) else (shutil.which("nvcc") or "nvcc")


def _cxx():
    return shutil.which("g++") or "g++"


def _common_flags():
    return ARCH + ["-O3", "-std=c++17", "-lineinfo", "-Xcompiler", "-fPIC", "-Xcompiler", "-ffp-contract=off",
                   "-I" + INCLUDE, "-I" + CSRC]


def _jobs():
    nv = _nvcc()
    jobs = []
    for s in SYSTEMS:
        for n in DEGREES:
            d = ["-DADERDG_SYS=%d" % s, "-DADERDG_N=%d" % n]
            jobs.append(([nv] + _common_flags() + d + ["-c", os.path.join(CSRC, "predictor_tu.cu")],
                         "pred_%d_%d.o" % (s, n)))
            jobs.append(([nv] + _common_flags() + ["--fmad=false"] + d + ["-c", os.path.join(CSRC, "exact_tu.cu")],
                         "exact_%d_%d.o" % (s, n)))
            # the tuner's candidates (aderdg/tuner.py): FP32 predictor shapes and K3 CTA sizes
            jobs.append(([nv] + _common_flags() + ["--fmad=false"] + d + ["-c", os.path.join(CSRC, "cells_var_tu.cu")],
                         "cellsvar_%d_%d.o" % (s, n)))
            for var in range(1, PRED_VARIANTS):
                jobs.append(([nv] + _common_flags() + d + ["-DADERDG_VAR=%d" % var, "-c",
                                                          os.path.join(CSRC, "predictor_var_tu.cu")],
                             "predvar_%d_%d_%d.o" % (s, n, var)))
    for src in ("registry.cu", "api.cu", "probe.cu", "batch.cu"):
        jobs.append(([nv] + _common_flags() + ["-c", os.path.join(CSRC, src)], src.replace(".cu", ".o")))
    jobs.append(([nv] + _common_flags() + ["--fmad=false", "-c", os.path.join(CSRC, "noalloc.cu")], "noalloc.o"))
    jobs.append(([nv] + _common_flags() + ["--fmad=false", "-c", os.path.join(CSRC, "initial.cu")], "initial.o"))
    jobs.append(([nv] + _common_flags() + ["--fmad=false", "-c", os.path.join(CSRC, "output.cu")], "output.o"))
    jobs.append((["g++", "-O2", "-std=c++17", "-fPIC", "-ffp-contract=off", "-I" + INCLUDE, "-c",
                  os.path.join(CSRC, "setup.cpp")], "setup.o"))
    return jobs


def _stamp():
    h = hashlib.sha256()
    for d in (CSRC, INCLUDE, os.path.join(PKG_ROOT, "host")):
        for f in sorted(os.listdir(d)):
            p = os.path.join(d, f)
            if os.path.isfile(p):
                h.update(f.encode())
                with open(p, "rb") as fh:
                    h.update(fh.read())
    h.update(repr(_jobs()).encode())
    return h.hexdigest()


def build(force=False, verbose=False, max_workers=None):
    """Compile every kernel family and link libaderdg_gpu.so; returns its path."""
    os.makedirs(BUILD_DIR, exist_ok=True)
    stamp_path = os.path.join(BUILD_DIR, "stamp.txt")
    stamp = _stamp()
    if not force and os.path.exists(LIB_PATH) and os.path.exists(stamp_path):
        with open(stamp_path) as fh:
            if fh.read().strip() == stamp:
                return LIB_PATH
    jobs = _jobs()
    workers = max_workers or max(1, os.cpu_count() or 1)

    def run(job):
        cmd, obj = job
        out = os.path.join(BUILD_DIR, obj)
        r = subprocess.run(cmd + ["-o", out], capture_output=True, text=True)
        if r.returncode != 0:
            raise RuntimeError("compile failed: %s\n%s%s" % (" ".join(cmd), r.stdout, r.stderr))
        if verbose and (r.stdout or r.stderr):
            print(r.stdout + r.stderr)
        return out

    with concurrent.futures.ThreadPoolExecutor(max_workers=workers) as ex:
        objs = list(ex.map(run, jobs))
    link = [_nvcc()] + ARCH + ["-shared", "-o", LIB_PATH] + objs + ["-cudart", "static"]
    r = subprocess.run(link, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError("link failed: %s\n%s%s" % (" ".join(link), r.stdout, r.stderr))
    drv = [_cxx(), "-O2", "-std=c++17", "-I" + INCLUDE, os.path.join(PKG_ROOT, "host", "aderdg_driver.cpp"),
           "-o", DRIVER_PATH, "-L" + BUILD_DIR, "-laderdg_gpu", "-Wl,-rpath,$ORIGIN"]
    r = subprocess.run(drv, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError("driver build failed: %s\n%s%s" % (" ".join(drv), r.stdout, r.stderr))
    with open(stamp_path, "w") as fh:
        fh.write(stamp)
    return LIB_PATH


if __name__ == "__main__":
    print(build(force=True, verbose=True))
