"""CPU oracle for the lattice Boltzmann step -- TEST INFRASTRUCTURE, NOT PRODUCT CODE.

Only ``tests/``, ``__graft_entry__.smoke()`` and the ``cpu_baseline`` / ``--impl reference`` legs
of ``bench.py`` may import this package, and only as the checker (or the timed CPU baseline).  The
GPU library never imports, links or calls it.

``lbm_oracle.c`` restates the reference kernels of ``simulation/source/SimCalcFuncs.cu`` (D3Q27)
and the project's D2Q9 BGK step; this module binds it with ctypes on numpy arrays.  ``refkern``
(sub-module) drives the reference's own CUDA kernels, compiled from their sources into
``oracle/_ref/``, on a GPU.
"""
from __future__ import annotations

import ctypes
import os
import subprocess

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(HERE, "liblbm_oracle.so")

# D3Q27 tables (SimCalcFuncs.cu:12-14, Constants.cpp:6-7)
C27 = np.array(
    [[0, 0, 0], [-1, 0, 0], [0, -1, 0], [0, 0, -1], [0, 0, 1], [0, 1, 0], [1, 0, 0],
     [-1, -1, 0], [-1, 0, -1], [-1, 0, 1], [-1, 1, 0], [0, -1, -1], [0, -1, 1], [0, 1, -1],
     [0, 1, 1], [1, -1, 0], [1, 0, -1], [1, 0, 1], [1, 1, 0], [-1, -1, -1], [-1, -1, 1],
     [-1, 1, -1], [-1, 1, 1], [1, -1, -1], [1, -1, 1], [1, 1, -1], [1, 1, 1]], dtype=np.int32)
INV27 = np.array([0, 6, 5, 4, 3, 2, 1, 18, 17, 16, 15, 14, 13, 12, 11, 10, 9, 8, 7, 26, 25, 24,
                  23, 22, 21, 20, 19], dtype=np.int32)

# D2Q9 order shared with the GPU library
CX9 = np.array([0, 1, 0, -1, 0, 1, -1, -1, 1], dtype=np.int32)
CY9 = np.array([0, 0, 1, 0, -1, 1, 1, -1, -1], dtype=np.int32)
W9 = np.array([4 / 9] + [1 / 9] * 4 + [1 / 36] * 4, dtype=np.float64)
OPP9 = np.array([0, 3, 4, 1, 2, 7, 8, 5, 6], dtype=np.int32)

INTERNAL, REFLECTED, SOURCE = 1, 2, 4

REFL_DTYPE = np.dtype([("dirs", np.int32, (14,)), ("w", np.float32, (81,))])
assert REFL_DTYPE.itemsize == 380  # sizeof(ReflectionValues), LatticePoint.h:3-7


def build(force: bool = False) -> str:
    """Compile lbm_oracle.c with gcc + OpenMP (same recipe on x86_64 and aarch64)."""
    src = os.path.join(HERE, "lbm_oracle.c")
    if force or not os.path.exists(LIB_PATH) or os.path.getmtime(LIB_PATH) < os.path.getmtime(src):
        subprocess.check_call(["gcc", "-std=c11", "-O3", "-fPIC", "-shared", "-fopenmp",
                               "-ffp-contract=off", "-o", LIB_PATH, src, "-lm"])
    return LIB_PATH


_lib = None


def lib():
    global _lib
    if _lib is None:
        build()
        L = ctypes.CDLL(LIB_PATH)
        P = ctypes.c_void_p
        i, f, d = ctypes.c_int, ctypes.c_float, ctypes.c_double
        L.orc_d3q27_stream.argtypes = [i, i, i, P, P]
        L.orc_d3q27_collide.argtypes = [i, i, i, P, f]
        L.orc_d3q27_reflect.argtypes = [i, i, i, P, P, P, P, P, P, i]
        L.orc_d3q27_flow.argtypes = [i, i, i, P, P, P]
        L.orc_d3q27_run.argtypes = [i, i, i, P, P, P, P, f, P, i, i, P, i]
        L.orc_refl_get_dir.argtypes = [P, i]
        L.orc_refl_set_dir.argtypes = [P, i, i]
        L.orc_compress_ints.argtypes = [P, i, i]
        L.orc_compress_ints.restype = ctypes.c_uint
        for suf, real in (("f64", d), ("f32", f)):
            getattr(L, f"orc_d2q9_step_{suf}").argtypes = [i, i, i, P, real, real, real, real, real, P, P]
            getattr(L, f"orc_d2q9_run_{suf}").argtypes = [i, i, i, P, real, real, real, real, real, P, i]
            getattr(L, f"orc_d2q9_moments_{suf}").argtypes = [i, i, i, P, real, real, real, real, P, P, P, P]
            getattr(L, f"orc_d2q9_equilibrium_{suf}").argtypes = [i, i, P, P, P, P]
            getattr(L, f"orc_d2q9_conservation_{suf}").argtypes = [i, i, P, P, P]
        L.orc_num_threads.restype = i
        L.orc_set_num_threads.argtypes = [i]
        _lib = L
    return _lib


def _p(a):
    return None if a is None else a.ctypes.data_as(ctypes.c_void_p)


def _chk(rc, what):
    if rc != 0:
        raise RuntimeError(f"oracle {what} failed with {rc}")


def num_threads() -> int:
    return lib().orc_num_threads()


def set_num_threads(n: int) -> None:
    lib().orc_set_num_threads(int(n))


# ----------------------------------------------------------------------------------------------
# D3Q27 reference restatement.  Arrays are cell-major f[cell, 27] with cell = z + Z*(y + Y*x).
# ----------------------------------------------------------------------------------------------
def d3q27_stream(dims, f):
    X, Y, Z = dims
    f = np.ascontiguousarray(f, dtype=np.float32)
    out = np.empty_like(f)
    _chk(lib().orc_d3q27_stream(X, Y, Z, _p(f), _p(out)), "stream")
    return out


def d3q27_collide(dims, f, tau):
    X, Y, Z = dims
    f = np.array(f, dtype=np.float32, copy=True, order="C")
    _chk(lib().orc_d3q27_collide(X, Y, Z, _p(f), float(tau)), "collide")
    return f


def d3q27_reflect(dims, f, flags, tab_idx, tabs, force=None, force_mode=0):
    X, Y, Z = dims
    f = np.ascontiguousarray(f, dtype=np.float32)
    out = np.empty_like(f)
    flags = np.ascontiguousarray(flags, dtype=np.uint8)
    tab_idx = np.ascontiguousarray(tab_idx, dtype=np.int32)
    tabs = np.ascontiguousarray(tabs, dtype=REFL_DTYPE)
    _chk(lib().orc_d3q27_reflect(X, Y, Z, _p(f), _p(out), _p(flags), _p(tab_idx), _p(tabs),
                                 _p(force), int(force_mode)), "reflect")
    return out


def d3q27_flow(dims, f, flags, induced):
    X, Y, Z = dims
    f = np.array(f, dtype=np.float32, copy=True, order="C")
    flags = np.ascontiguousarray(flags, dtype=np.uint8)
    induced = np.ascontiguousarray(induced, dtype=np.float32)
    _chk(lib().orc_d3q27_flow(X, Y, Z, _p(f), _p(flags), _p(induced)), "flow")
    return f


def d3q27_run(dims, f, flags, tau, nsteps, order=0, tab_idx=None, tabs=None, induced=None,
              force=None, force_mode=0):
    X, Y, Z = dims
    f = np.array(f, dtype=np.float32, copy=True, order="C")
    flags = np.ascontiguousarray(flags, dtype=np.uint8)
    if tab_idx is not None:
        tab_idx = np.ascontiguousarray(tab_idx, dtype=np.int32)
        tabs = np.ascontiguousarray(tabs, dtype=REFL_DTYPE)
    if induced is not None:
        induced = np.ascontiguousarray(induced, dtype=np.float32)
    _chk(lib().orc_d3q27_run(X, Y, Z, _p(f), _p(flags), _p(tab_idx), _p(tabs), float(tau),
                             _p(induced), int(order), int(nsteps), _p(force), int(force_mode)), "run")
    return f


def refl_set_dir(rec, slot, d):
    """Pack direction d into slot of one REFL_DTYPE record (Lattice.cpp:450-463)."""
    buf = np.array([rec], dtype=REFL_DTYPE)
    lib().orc_refl_set_dir(_p(buf), int(slot), int(d))
    rec["dirs"][:] = buf[0]["dirs"]


def refl_get_dir(rec, slot):
    buf = np.array([rec], dtype=REFL_DTYPE)
    return lib().orc_refl_get_dir(_p(buf), int(slot))


def compress_ints(values, bit_length):
    a = np.ascontiguousarray(values, dtype=np.int32)
    return int(lib().orc_compress_ints(_p(a), len(a), int(bit_length)))


# ----------------------------------------------------------------------------------------------
# D2Q9.  SoA f[q, ny, nx]; flags[ny, nx] in {0 fluid, 1 wall, 2 moving wall}.
# ----------------------------------------------------------------------------------------------
def _real(dtype):
    return "f64" if np.dtype(dtype) == np.float64 else "f32"


def d2q9_equilibrium(rho, ux, uy, dtype=np.float64):
    ny, nx = np.shape(rho)
    rho = np.ascontiguousarray(rho, dtype=dtype)
    ux = np.ascontiguousarray(ux, dtype=dtype)
    uy = np.ascontiguousarray(uy, dtype=dtype)
    f = np.empty((9, ny, nx), dtype=dtype)
    _chk(getattr(lib(), f"orc_d2q9_equilibrium_{_real(dtype)}")(nx, ny, _p(rho), _p(ux), _p(uy), _p(f)), "eq")
    return f


def d2q9_run(f, flags, tau, nsteps, periodic=0, force=(0.0, 0.0), wall_velocity=(0.0, 0.0)):
    f = np.array(f, copy=True, order="C")
    _, ny, nx = f.shape
    flags = np.ascontiguousarray(flags, dtype=np.uint8)
    fn = getattr(lib(), f"orc_d2q9_run_{_real(f.dtype)}")
    _chk(fn(nx, ny, int(periodic), _p(flags), tau, force[0], force[1], wall_velocity[0],
            wall_velocity[1], _p(f), int(nsteps)), "d2q9 run")
    return f


def d2q9_step(f, flags, tau, periodic=0, force=(0.0, 0.0), wall_velocity=(0.0, 0.0), out=None):
    f = np.ascontiguousarray(f)
    _, ny, nx = f.shape
    out = np.empty_like(f) if out is None else out
    flags = np.ascontiguousarray(flags, dtype=np.uint8)
    fn = getattr(lib(), f"orc_d2q9_step_{_real(f.dtype)}")
    _chk(fn(nx, ny, int(periodic), _p(flags), tau, force[0], force[1], wall_velocity[0],
            wall_velocity[1], _p(f), _p(out)), "d2q9 step")
    return out


def d2q9_moments(f, flags, periodic=0, force=(0.0, 0.0), wall_velocity=(0.0, 0.0)):
    f = np.ascontiguousarray(f)
    _, ny, nx = f.shape
    flags = np.ascontiguousarray(flags, dtype=np.uint8)
    rho = np.empty((ny, nx), dtype=f.dtype)
    ux = np.empty_like(rho)
    uy = np.empty_like(rho)
    fn = getattr(lib(), f"orc_d2q9_moments_{_real(f.dtype)}")
    _chk(fn(nx, ny, int(periodic), _p(flags), force[0], force[1], wall_velocity[0],
            wall_velocity[1], _p(f), _p(rho), _p(ux), _p(uy)), "moments")
    return rho, ux, uy


def d2q9_conservation(f, flags):
    f = np.ascontiguousarray(f)
    _, ny, nx = f.shape
    flags = np.ascontiguousarray(flags, dtype=np.uint8)
    out = np.zeros(3, dtype=np.float64)
    fn = getattr(lib(), f"orc_d2q9_conservation_{_real(f.dtype)}")
    _chk(fn(nx, ny, _p(flags), _p(f), _p(out)), "conservation")
    return out


# ----------------------------------------------------------------------------- seeded channel geometry
_M64 = (1 << 64) - 1


class _SplitMix64:
    """SplitMix64 (Steele, Lea, Flood 2014), the generator behind the library's seeded geometry;
    restated here so that the CPU baseline builds the benchmark channel without the GPU library."""

    def __init__(self, seed):
        self.s = int(seed) & _M64

    def next(self):
        self.s = (self.s + 0x9E3779B97F4A7C15) & _M64
        z = self.s
        z = ((z ^ (z >> 30)) * 0xBF58476D1CE4E5B9) & _M64
        z = ((z ^ (z >> 27)) * 0x94D049BB133111EB) & _M64
        return z ^ (z >> 31)

    def u01(self):
        return float(self.next() >> 11) * (1.0 / 9007199254740992.0)


def channel_flags(nx, ny, ndisks, rmin, rmax, seed):
    """D2Q9 channel flags: walls on rows 0 and ny-1, `ndisks` non-overlapping disks (x-periodic
    distance) with centres uniform in [0,nx) x [0,ny) and radius uniform in [rmin, rmax], placed by
    rejection in SplitMix64 order; a cell is solid when its centre lies inside a disk (x wraps).
    The same flags as the library's lbm_gen_channel for the same arguments."""
    flags = np.zeros((ny, nx), np.uint8)
    flags[0, :] = 1
    flags[-1, :] = 1
    rng = _SplitMix64(seed)
    rmin32, span32 = float(np.float32(rmin)), float(np.float32(rmax)) - float(np.float32(rmin))
    placed = []
    for _ in range(1000000):
        if len(placed) >= ndisks:
            break
        d = (rng.u01() * nx, rng.u01() * ny, rmin32 + rng.u01() * span32)
        ok = True
        for p in placed:
            dx = abs(d[0] - p[0])
            dx = min(dx, nx - dx)
            dy = d[1] - p[1]
            if dx * dx + dy * dy < (d[2] + p[2]) * (d[2] + p[2]):
                ok = False
                break
        if ok:
            placed.append(d)
    if len(placed) < ndisks:
        raise ValueError(f"could not place {ndisks} non-overlapping disks")
    for cx, cy, r in placed:
        y0, y1 = max(0, int(np.floor(cy - r - 1.0))), min(ny - 1, int(np.ceil(cy + r + 1.0)))
        x0, x1 = int(np.floor(cx - r - 1.0)), int(np.ceil(cx + r + 1.0))
        ys = np.arange(y0, y1 + 1)
        xs = np.arange(x0, x1 + 1)
        dy = (ys + 0.5) - cy
        dx = (xs + 0.5) - cx
        inside = dx[None, :] ** 2 + dy[:, None] ** 2 <= r * r
        yy, xx = np.nonzero(inside)
        flags[ys[yy], np.mod(xs[xx], nx)] = 1
    return flags
