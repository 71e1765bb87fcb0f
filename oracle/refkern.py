"""The reference's own CUDA kernels as a GPU oracle -- TEST INFRASTRUCTURE, NOT PRODUCT CODE.

Recipe (``build()``):
  1. Where the reference sources are readable (the directory given to build(), else the
     REFERENCE_ROOT environment variable; there is no built-in default), compile
     simulation/source/SimCalcFuncs.cu with simulation/source/FlowCriterion.cu force-included as one
     translation unit, for sm_103a, into oracle/_ref/ref_kernels.cubin.  The sources are compiled
     where they lie; nothing is copied.  (The reference builds these two files with separable
     compilation into a static library; one translation unit gives the same kernels without a
     device-link step.)  The cubin is device code only, so it also runs where the sources are absent.
  2. Compile oracle/ref_harness.cpp (our driver-API harness) into oracle/_ref/libref_harness.so.

``run()`` drives the kernels in the order of the reference's Lattice methods on LatticePoint
records and returns the records afterwards.
"""
from __future__ import annotations

import ctypes
import os
import shutil
import subprocess

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
REF_DIR = os.path.join(HERE, "_ref")
CUBIN = os.path.join(REF_DIR, "ref_kernels.cubin")
HARNESS = os.path.join(REF_DIR, "libref_harness.so")

LATTICE_POINT = np.dtype({
    "names": ["x", "y", "z", "f", "isReflected", "isInternal", "reflections", "d_reflections"],
    "formats": [np.int32, np.int32, np.int32, (np.float32, (27,)), np.bool_, np.bool_, np.uint64, np.uint64],
    "offsets": [0, 4, 8, 12, 120, 121, 128, 136], "itemsize": 144})
REFLECTION_VALUES = np.dtype([("dirs", np.int32, (14,)), ("w", np.float32, (81,))])


def _nvcc():
    for c in (os.environ.get("NVCC"), "/usr/local/cuda/bin/nvcc", shutil.which("nvcc")):
        if c and os.path.exists(c):
            return c
    raise RuntimeError("nvcc not found")


def build_cubin(reference_root=None, force=False) -> bool:
    """Compile the reference kernels from the sources under `reference_root` (or $REFERENCE_ROOT).
    Without either, or where the sources are absent, an existing cubin is kept as it is."""
    root = reference_root or os.environ.get("REFERENCE_ROOT")
    if not root:
        return os.path.exists(CUBIN)
    src = os.path.join(root, "simulation", "source", "SimCalcFuncs.cu")
    flow = os.path.join(root, "simulation", "source", "FlowCriterion.cu")
    inc = os.path.join(root, "simulation", "include")
    if not os.path.exists(src):
        return os.path.exists(CUBIN)
    if os.path.exists(CUBIN) and not force and os.path.getmtime(CUBIN) > os.path.getmtime(src):
        return True
    os.makedirs(REF_DIR, exist_ok=True)
    subprocess.check_call([_nvcc(), "-cubin", "-gencode", "arch=compute_103a,code=sm_103a", "-O3",
                           "-I", inc, "-include", flow, src, "-o", CUBIN])
    return True


def build_harness(force=False) -> bool:
    src = os.path.join(HERE, "ref_harness.cpp")
    if os.path.exists(HARNESS) and not force and os.path.getmtime(HARNESS) > os.path.getmtime(src):
        return True
    os.makedirs(REF_DIR, exist_ok=True)
    tmp = HARNESS + ".tmp"
    subprocess.check_call([_nvcc(), "-O2", "-std=c++17", "-shared", "-Xcompiler", "-fPIC", src, "-o", tmp,
                           "-lcuda"])
    os.replace(tmp, HARNESS)
    return True


def build(reference_root=None, force=False) -> bool:
    ok = build_cubin(reference_root, force)
    build_harness(force)
    return ok


def available() -> bool:
    return os.path.exists(CUBIN)


_h = None


def harness():
    global _h
    if _h is None:
        build_harness()
        L = ctypes.CDLL(HARNESS)
        P = ctypes.c_void_p
        L.rk_error.restype = ctypes.c_char_p
        L.rk_last_seconds.restype = ctypes.c_double
        L.rk_init.argtypes = [ctypes.c_char_p]
        L.rk_run.argtypes = [ctypes.c_int, ctypes.c_int, ctypes.c_int, P, P, P, ctypes.c_int, ctypes.c_float,
                             ctypes.c_char_p, ctypes.c_int, ctypes.c_int, P, P, P]
        if L.rk_init(CUBIN.encode()) != 0:
            raise RuntimeError("reference kernels: " + L.rk_error().decode())
        _h = L
    return _h


def _p(a):
    return None if a is None else ctypes.c_void_p(a.ctypes.data)


def run(dims, points, ops, nsteps=1, tau=1.0, tab_cells=None, tab_records=None, flow_criterion=0,
        induced=None, force=None, threads=(1, 1, 1)):
    """Run the reference kernels on LatticePoint records (host index z + Z*(y + Y*x)).
    ops: pass letters per step, e.g. "SC" (Lattice::simulateLattice) or "SRCF" (CLI loop).
    force: None, or a float32[3] start value updated in place."""
    X, Y, Z = dims
    pts = np.array(points, dtype=LATTICE_POINT, copy=True)
    cells = np.ascontiguousarray([] if tab_cells is None else tab_cells, dtype=np.int32)
    recs = np.ascontiguousarray(np.zeros(0, REFLECTION_VALUES) if tab_records is None else tab_records,
                                dtype=REFLECTION_VALUES)
    ind = np.ascontiguousarray(np.zeros(27) if induced is None else induced, dtype=np.float32)
    thr = np.ascontiguousarray(threads, dtype=np.int32)
    rc = harness().rk_run(X, Y, Z, _p(pts), _p(cells) if cells.size else None, _p(recs) if recs.size else None,
                          int(cells.size), float(tau), ops.encode(), int(nsteps), int(flow_criterion), _p(ind),
                          _p(force), _p(thr))
    if rc != 0:
        raise RuntimeError("reference kernels: " + harness().rk_error().decode())
    return pts


def last_seconds():
    """Seconds of the last run()'s step loop."""
    return float(harness().rk_last_seconds())
