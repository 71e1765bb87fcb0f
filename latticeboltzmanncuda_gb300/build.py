"""Build liblbm_gb300.so in-tree: every CUDA / C++ source of csrc/ compiled by nvcc for sm_103a only,
in parallel, then linked into one shared library with the C ABI of include/lbm_capi.h.

    python -m latticeboltzmanncuda_gb300.build [--force] [-v]

The kernels' index arithmetic is checked on the CPU instead of by a bounds-checked device build:
tests/test_index_bounds.py replays every launch shape's addressing against the buffer sizes.
"""
from __future__ import annotations

import argparse
import concurrent.futures as cf
import hashlib
import os
import shutil
import subprocess
import sys

PKG = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(PKG)
CSRC = os.path.join(PKG, "csrc")
INCLUDE = os.path.join(ROOT, "include")
OUT_DIR = os.path.join(PKG, "_build")
LIB = os.path.join(PKG, "liblbm_gb300.so")
COMPAT = os.path.join(PKG, "compat")
COMPAT_LIB = os.path.join(PKG, "liblbm_compat.so")
CLI = os.path.join(PKG, "bin", "LatticeBoltzmannCuda")

ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]
SOURCES = ["common.cu", "capi.cu", "d2q9.cu", "d3q27.cu", "geometry.cpp", "mesh.cpp", "noalloc.cu", "batch.cu",
           "server.cpp", "checkpoint.cpp"]


def nvcc() -> str:
    for cand in (os.environ.get("NVCC"), "/usr/local/cuda/bin/nvcc", shutil.which("nvcc")):
        if cand and os.path.exists(cand):
            return cand
    raise RuntimeError("nvcc not found: the CUDA toolkit is required to build liblbm_gb300.so")


def _flags():
    # host code: no floating-point contraction, so x86-64 and aarch64 builds give the same results
    return ["-O3", "-std=c++17", "-lineinfo", "-Xcompiler", "-fPIC,-fvisibility=hidden,-ffp-contract=off",
            "-I", INCLUDE, "-I", CSRC, "--expt-relaxed-constexpr"]


def _digest(paths, extra: str) -> str:
    h = hashlib.sha256(extra.encode())
    for p in sorted(paths):
        with open(p, "rb") as fh:
            h.update(p.encode())
            h.update(fh.read())
    return h.hexdigest()


def _inputs():
    hdrs = [os.path.join(CSRC, f) for f in os.listdir(CSRC) if f.endswith((".h", ".cuh"))]
    hdrs.append(os.path.join(INCLUDE, "lbm_capi.h"))
    return [os.path.join(CSRC, s) for s in SOURCES] + hdrs


def build(force: bool = False, verbose: bool = False) -> str:
    os.makedirs(OUT_DIR, exist_ok=True)
    stamp = os.path.join(OUT_DIR, "stamp")
    digest = _digest(_inputs(), " ".join(_flags()) + " ".join(ARCH))
    if not force and os.path.exists(LIB) and os.path.exists(stamp):
        with open(stamp) as fh:
            if fh.read().strip() == digest:
                build_compat()
                return LIB
    cc = nvcc()
    flags = _flags()

    def compile_one(src):
        obj = os.path.join(OUT_DIR, os.path.basename(src) + ".o")
        cmd = [cc, *ARCH, *flags, "-c", os.path.join(CSRC, src), "-o", obj]
        if src.endswith(".cpp"):
            cmd = [cc, *flags, "-x", "c++", "-c", os.path.join(CSRC, src), "-o", obj]
        r = subprocess.run(cmd, capture_output=True, text=True)
        if r.returncode != 0:
            raise RuntimeError(f"nvcc failed on {src}:\n{r.stdout}\n{r.stderr}")
        if verbose and (r.stdout or r.stderr):
            print(r.stdout, r.stderr, file=sys.stderr)
        return obj

    with cf.ThreadPoolExecutor(max_workers=min(len(SOURCES), os.cpu_count() or 4)) as ex:
        objs = list(ex.map(compile_one, SOURCES))
    tmp = LIB + ".tmp"
    cmd = [cc, *ARCH, "-shared", "-o", tmp, *objs, "-Xcompiler", "-fvisibility=hidden"]
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError(f"link failed:\n{r.stdout}\n{r.stderr}")
    os.replace(tmp, LIB)
    build_compat(force=True)
    with open(stamp, "w") as fh:
        fh.write(digest)
    return LIB


def _cxx() -> str:
    for cand in (os.environ.get("CXX"), shutil.which("g++"), shutil.which("c++")):
        if cand:
            return cand
    raise RuntimeError("no C++ compiler found for the compatibility layer")


def cuda_dirs():
    """(include dir, library dir holding libcudart.so) of the CUDA toolkit that nvcc belongs to."""
    root = os.path.dirname(os.path.dirname(os.path.realpath(nvcc())))
    lib = os.path.join(root, "lib64")
    if not os.path.exists(os.path.join(lib, "libcudart.so")):
        import glob
        found = glob.glob(os.path.join(root, "targets", "*", "lib", "libcudart.so"))
        lib = os.path.dirname(found[0]) if found else lib
    return os.path.join(root, "include"), lib


def build_compat(force: bool = False) -> str:
    """The reference's C++ API (compat/include, compat/src/compat.cpp) as liblbm_compat.so on top of
    liblbm_gb300.so, and the reference's command line as bin/LatticeBoltzmannCuda."""
    srcs = [os.path.join(COMPAT, "src", f) for f in ("compat.cpp", "LatticeBoltzmannCuda.cpp")]
    hdrs = [os.path.join(COMPAT, "include", f) for f in sorted(os.listdir(os.path.join(COMPAT, "include")))]
    stamp = os.path.join(OUT_DIR, "compat.stamp")
    digest = _digest(srcs + hdrs + [os.path.join(INCLUDE, "lbm_capi.h")], "compat")
    if not force and os.path.exists(COMPAT_LIB) and os.path.exists(CLI) and os.path.exists(stamp):
        with open(stamp) as fh:
            if fh.read().strip() == digest:
                return COMPAT_LIB
    cuda_inc, cuda_lib = cuda_dirs()
    common = ["-std=c++17", "-O2", "-fPIC", "-ffp-contract=off", "-Wall", "-I", os.path.join(COMPAT, "include"),
              "-I", INCLUDE, "-I", cuda_inc]
    # the layer itself calls the CUDA runtime (device ReflectionData objects of the reference's launcher)
    cudart = ["-L", cuda_lib, "-lcudart", f"-Wl,-rpath,{cuda_lib}"]
    os.makedirs(os.path.dirname(CLI), exist_ok=True)
    steps = [
        [_cxx(), *common, "-shared", srcs[0], "-o", COMPAT_LIB + ".tmp", "-L", PKG, "-llbm_gb300",
         "-Wl,-rpath,$ORIGIN", *cudart],
        [_cxx(), *common, srcs[1], "-o", CLI + ".tmp", "-L", PKG, "-llbm_compat", "-llbm_gb300",
         "-Wl,-rpath,$ORIGIN/..", *cudart],
    ]
    for cmd, out in zip(steps, (COMPAT_LIB, CLI)):
        if cmd is steps[1]:
            os.replace(COMPAT_LIB + ".tmp", COMPAT_LIB)
        r = subprocess.run(cmd, capture_output=True, text=True)
        if r.returncode != 0:
            raise RuntimeError(f"compatibility layer build failed:\n{' '.join(cmd)}\n{r.stdout}\n{r.stderr}")
    os.replace(CLI + ".tmp", CLI)
    with open(stamp, "w") as fh:
        fh.write(digest)
    return COMPAT_LIB


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--force", action="store_true")
    ap.add_argument("-v", "--verbose", action="store_true")
    a = ap.parse_args()
    print(build(force=a.force, verbose=a.verbose))


if __name__ == "__main__":
    main()
