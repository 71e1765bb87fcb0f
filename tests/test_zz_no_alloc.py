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


def _state(nx, ny, seed, steps=9):
    flags, rho, ux, uy = domain(nx, ny, seed)
    with lbm.Lattice(nx, ny, dtype="f64", tau=0.7, wall_velocity=(0.03, 0, 0)) as L:
        L.set_flags(flags)
        L.init_equilibrium(rho, ux, uy)
        L.step(steps)
        return flags, L.conservation()[:3], L.retrieve_populations(np.float64)


def test_noalloc_at_the_row_limit():
    """ny == LBM_NOALLOC_MAX_ROWS fills every partial triple of the fixed array."""
    torch = pytest.importorskip("torch")
    nx, ny = 4, capi.NOALLOC_MAX_ROWS
    flags = np.zeros((ny, nx), np.uint8)
    flags[:, 0] = lbm.WALL
    rng = np.random.default_rng(11)
    with lbm.Lattice(nx, ny, dtype="f64", tau=0.8, periodic=2) as L:
        L.set_flags(flags)
        L.init_equilibrium((1 + 0.01 * rng.standard_normal((ny, nx))).astype(np.float32),
                           (0.02 * rng.standard_normal((ny, nx))).astype(np.float32),
                           (0.02 * rng.standard_normal((ny, nx))).astype(np.float32))
        L.step(5)
        want = L.conservation()[:3]
        host = L.retrieve_populations(np.float64)
    dev = torch.device("cuda", 0)
    f_dev = torch.from_numpy(host).to(dev).contiguous()
    flags_dev = torch.from_numpy(flags).to(dev)
    out = torch.full((3,), float("nan"), dtype=torch.float64, device=dev)
    stream = torch.cuda.current_stream(dev).cuda_stream
    assert noalloc(f_dev, capi.F64, flags_dev, nx, ny, nx, out, stream) == capi.OK, capi.last_thread_error()
    torch.cuda.synchronize(dev)
    got = out.cpu().numpy()
    scale = np.array([abs(want[0]), abs(want[0]) * 1e-3, abs(want[0]) * 1e-3])
    assert np.all(np.abs(got - want) <= 1e-12 * scale), (got, want)


def test_noalloc_two_calls_in_one_stream_keep_their_own_results():
    """Calls queued back to back on one stream share the fixed array but are ordered, so each gives
    the sums of its own inputs."""
    torch = pytest.importorskip("torch")
    dev = torch.device("cuda", 0)
    (fa, wa, ha), (fb, wb, hb) = _state(90, 61, 21), _state(57, 130, 22)
    stream = torch.cuda.current_stream(dev).cuda_stream
    bufs = []
    for flags, host in ((fa, ha), (fb, hb)):
        bufs.append((torch.from_numpy(host).to(dev).contiguous(), torch.from_numpy(flags).to(dev),
                     torch.full((3,), float("nan"), dtype=torch.float64, device=dev), flags.shape))
    for f_dev, flags_dev, out, (ny, nx) in bufs:
        assert noalloc(f_dev, capi.F64, flags_dev, nx, ny, nx, out, stream) == capi.OK, capi.last_thread_error()
    torch.cuda.synchronize(dev)
    for (_, _, out, _), want in zip(bufs, (wa, wb)):
        got = out.cpu().numpy()
        scale = np.array([abs(want[0]), abs(want[0]) * 1e-3, abs(want[0]) * 1e-3])
        assert np.all(np.abs(got - want) <= 1e-12 * scale), (got, want)
