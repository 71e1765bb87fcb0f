"""lbm_d2q9_conservation_noalloc: the allocation-free conservation sums, for callers that own all
of their device memory and cannot let the library allocate (fixed device budgets, latency-bound
loops where cudaMalloc would synchronise the device).

The caller's buffers here are torch tensors, as a caller that manages its own device memory would
hold them; the entry point is called through the C ABI, twice in a row on the same buffers, and
compared with the existing lbm_conservation of the same state (FP64 storage: 1e-12 relative;
FP32 storage: 1e-6 relative, the tolerance of the conservation tests).
"""
import ctypes

import numpy as np
import pytest

import latticeboltzmanncuda_gb300 as lbm
from latticeboltzmanncuda_gb300 import capi

pytestmark = pytest.mark.gpu


def domain(nx, ny, seed):
    flags = lbm.gen_cavity(nx, ny)
    flags[ny // 3: ny // 3 + 5, nx // 2: nx // 2 + 7] = lbm.WALL
    rng = np.random.default_rng(seed)
    rho = (1 + 0.01 * rng.standard_normal((ny, nx))).astype(np.float32)
    ux = (0.02 * rng.standard_normal((ny, nx))).astype(np.float32)
    uy = (0.02 * rng.standard_normal((ny, nx))).astype(np.float32)
    return flags, rho, ux, uy


def noalloc(f_dev, dtype, flags_dev, nx, ny, row_pitch, out_dev, stream):
    return capi.lib().lbm_d2q9_conservation_noalloc(ctypes.c_void_p(f_dev.data_ptr()), dtype,
                                                    ctypes.c_void_p(flags_dev.data_ptr()), nx, ny, row_pitch,
                                                    ctypes.c_void_p(out_dev.data_ptr()), ctypes.c_void_p(stream))


@pytest.mark.parametrize("store,rtol", [("f64", 1e-12), ("f32", 1e-6)])
def test_noalloc_matches_lbm_conservation_twice(store, rtol):
    torch = pytest.importorskip("torch")
    nx, ny = 150, 97
    flags, rho, ux, uy = domain(nx, ny, 3)
    with lbm.Lattice(nx, ny, dtype=store, tau=0.6, wall_velocity=(0.04, 0, 0)) as L:
        L.set_flags(flags)
        L.init_equilibrium(rho, ux, uy)
        L.step(25)
        want = L.conservation()[:3]
        host = L.retrieve_populations(np.float64 if store == "f64" else np.float32)
    dev = torch.device("cuda", 0)
    # caller-owned buffers, with a row pitch wider than nx
    pitch = nx + 10
    f_dev = torch.zeros((9, ny, pitch), dtype=torch.float64 if store == "f64" else torch.float32, device=dev)
    f_dev[:, :, :nx] = torch.from_numpy(host).to(dev)
    flags_dev = torch.from_numpy(np.ascontiguousarray(flags)).to(dev)
    out = torch.empty(3, dtype=torch.float64, device=dev)
    stream = torch.cuda.current_stream(dev).cuda_stream
    dt = capi.F64 if store == "f64" else capi.F32
    scale = np.array([abs(want[0]), abs(want[0]) * 1e-3, abs(want[0]) * 1e-3])
    for _ in range(2):
        out.fill_(float("nan"))  # each call must write every component
        rc = noalloc(f_dev, dt, flags_dev, nx, ny, pitch, out, stream)
        assert rc == capi.OK, capi.last_thread_error()
        torch.cuda.synchronize(dev)
        got = out.cpu().numpy()
        assert np.all(np.abs(got - want) <= rtol * scale), (got, want)


def test_noalloc_rejects_too_many_rows_and_bad_arguments():
    torch = pytest.importorskip("torch")
    dev = torch.device("cuda", 0)
    f_dev = torch.zeros(9 * 8, dtype=torch.float32, device=dev)
    flags_dev = torch.zeros(8, dtype=torch.uint8, device=dev)
    out = torch.zeros(3, dtype=torch.float64, device=dev)
    # ny beyond the rows the fixed scratch array holds: rejected before any launch
    rc = noalloc(f_dev, capi.F32, flags_dev, 1, 32769, 1, out, 0)
    assert rc == capi.ERR_INVALID and "maximum" in capi.last_thread_error()
    assert noalloc(f_dev, 7, flags_dev, 8, 1, 8, out, 0) == capi.ERR_INVALID
    assert noalloc(f_dev, capi.F32, flags_dev, 8, 1, 4, out, 0) == capi.ERR_INVALID
