"""CPU-side checks of the C ABI: the library builds and loads, exports every symbol that
include/lbm_capi.h declares, validates arguments without touching a GPU, and the seeded geometry
generators are deterministic and meet their contracts."""
import ctypes
import os
import re
import subprocess

import numpy as np
import pytest

import latticeboltzmanncuda_gb300 as lbm
from latticeboltzmanncuda_gb300 import capi

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def declared_symbols():
    names = set()
    for h in os.listdir(os.path.join(ROOT, "include")):
        if h.endswith(".h"):
            txt = open(os.path.join(ROOT, "include", h)).read()
            names |= set(re.findall(r"LBM_API\s+[\w\s\*]+?\b(lbm_\w+)\s*\(", txt))
    return names


def test_library_exports_every_declared_symbol():
    L = capi.lib()
    names = declared_symbols()
    assert len(names) >= 25
    missing = [n for n in names if not hasattr(L, n)]
    assert not missing, missing
    bound = {n for n, _, _ in capi.SIGNATURES}
    assert names <= bound | {n for n in names if n.startswith(("lbm_batch", "lbm_server", "lbm_autotune", "lbm_obj", "lbm_mesh", "lbm_refl", "lbm_d2q9"))}


def test_struct_layouts(tmp_path):
    """ctypes mirrors of lbm_desc / lbm_info match the C compiler's layout of the header."""
    src = tmp_path / "layout.c"
    src.write_text('#include <stdio.h>\n#include <stddef.h>\n#include "lbm_capi.h"\n'
                   'int main(void){printf("%zu %zu %zu %zu %zu\\n", sizeof(lbm_desc), '
                   'offsetof(lbm_desc, tau), offsetof(lbm_desc, stream), sizeof(lbm_info), '
                   'offsetof(lbm_info, block_threads)); return 0;}\n')
    exe = tmp_path / "layout"
    subprocess.check_call(["gcc", "-I", os.path.join(ROOT, "include"), str(src), "-o", str(exe)])
    got = [int(v) for v in subprocess.check_output([str(exe)]).split()]
    assert got == [ctypes.sizeof(capi.Desc), capi.Desc.tau.offset, capi.Desc.stream.offset,
                   ctypes.sizeof(capi.Info), capi.Info.block_threads.offset]
    assert capi.LATTICE_POINT.itemsize == 144
    assert capi.LATTICE_POINT.fields["f"][1] == 12
    assert capi.REFLECTION_VALUES.itemsize == 380


def test_status_strings():
    L = capi.lib()
    assert L.lbm_status_string(capi.OK) == b"ok"
    assert L.lbm_status_string(capi.ERR_BUDGET).startswith(b"over")


def test_create_rejects_bad_descriptors_before_touching_the_gpu():
    L = capi.lib()
    ctx = ctypes.c_void_p()
    d = capi.Desc()
    L.lbm_desc_init(ctypes.byref(d))
    for field, value in (("mode", 7), ("dtype", 9), ("nx", 0), ("tau", 0.5), ("periodic", 4)):
        d2 = capi.Desc.from_buffer_copy(d)
        setattr(d2, field, value)
        assert L.lbm_create(ctypes.byref(d2), ctypes.byref(ctx)) == capi.ERR_INVALID
        assert capi.last_thread_error()
    d3 = capi.Desc.from_buffer_copy(d)
    d3.mode, d3.dtype = capi.D3Q27_REF, capi.F16S
    assert L.lbm_create(ctypes.byref(d3), ctypes.byref(ctx)) == capi.ERR_UNSUPPORTED
    assert L.lbm_step(None, 1) == capi.ERR_INVALID


def test_no_gpu_fails_loudly(gpu_available):
    if gpu_available:
        pytest.skip("a GPU is present")
    with pytest.raises(lbm.LBMError):
        lbm.Lattice(8, 8)


def test_gen_channel_contract():
    nx, ny, nd = 1024, 256, 16
    f1, disks = lbm.gen_channel(nx, ny, nd, 4, 10, 5)
    f2, _ = lbm.gen_channel(nx, ny, nd, 4, 10, 5)
    f3, _ = lbm.gen_channel(nx, ny, nd, 4, 10, 6)
    assert np.array_equal(f1, f2) and not np.array_equal(f1, f3)
    assert np.all(f1[0] == lbm.WALL) and np.all(f1[-1] == lbm.WALL)
    assert set(np.unique(f1)) <= {0, 1}
    assert disks.shape == (nd, 3)
    assert np.all((disks[:, 2] >= 4) & (disks[:, 2] <= 10))
    for i in range(nd):
        for j in range(i + 1, nd):
            dx = abs(disks[i, 0] - disks[j, 0])
            dx = min(dx, nx - dx)
            assert np.hypot(dx, disks[i, 1] - disks[j, 1]) >= disks[i, 2] + disks[j, 2] - 1e-4
    # every disk centre cell is solid, and the rasterisation matches the centre rule
    yy, xx = np.mgrid[0:ny, 0:nx]
    want = np.zeros((ny, nx), bool)
    want[0] = want[-1] = True
    for cx, cy, r in disks.astype(np.float64):
        dx = np.abs(xx + 0.5 - cx)
        dx = np.minimum(dx, nx - dx)
        want |= dx * dx + (yy + 0.5 - cy) ** 2 <= r * r + 1e-3
    assert np.mean(want == (f1 != 0)) > 0.9999


def test_gen_cavity_and_fraction():
    f = lbm.gen_cavity(32, 16)
    assert np.all(f[-1] == lbm.MOVING_WALL)
    assert np.all(f[0] == lbm.WALL) and np.all(f[:-1, 0] == lbm.WALL) and np.all(f[:-1, -1] == lbm.WALL)
    assert np.all(f[1:-1, 1:-1] == lbm.FLUID)
    g, ach = lbm.gen_disks_fraction(f, 0.2, 2, 4, 11)
    assert ach >= 0.2 and abs(ach - np.mean(g != 0)) < 1e-6
    assert np.all(g[-1] == lbm.MOVING_WALL)


def test_gen_rejects_impossible_packing():
    with pytest.raises(lbm.LBMError):
        lbm.gen_channel(64, 16, 500, 8, 8, 1)


def test_server_struct_layouts(tmp_path):
    """ctypes mirrors of the serving structs match the C compiler's layout of the header."""
    src = tmp_path / "srv.c"
    src.write_text('#include <stdio.h>\n#include <stddef.h>\n#include "lbm_capi.h"\n'
                   'int main(void){printf("%zu %zu %zu %zu %zu %zu %zu\\n", sizeof(lbm_server_config), '
                   'sizeof(lbm_request), offsetof(lbm_request, flags), offsetof(lbm_request, arrival), '
                   'sizeof(lbm_request_result), sizeof(lbm_server_stats), offsetof(lbm_server_stats, peak_slots));'
                   ' return 0;}\n')
    exe = tmp_path / "srv"
    subprocess.check_call(["gcc", "-I", os.path.join(ROOT, "include"), str(src), "-o", str(exe)])
    got = [int(v) for v in subprocess.check_output([str(exe)]).split()]
    assert got == [ctypes.sizeof(capi.ServerConfig), ctypes.sizeof(capi.Request), capi.Request.flags.offset,
                   capi.Request.arrival.offset, ctypes.sizeof(capi.RequestResult), ctypes.sizeof(capi.ServerStats),
                   capi.ServerStats.peak_slots.offset]


def test_server_rejects_bad_configuration():
    L = capi.lib()
    cfg = capi.ServerConfig()
    L.lbm_server_config_init(ctypes.byref(cfg))
    assert cfg.round_steps > 0 and cfg.budget_bytes == 150 * 10 ** 9
    srv = ctypes.c_void_p()
    for field, value in (("budget_bytes", 0), ("round_steps", 0), ("max_slots", -1), ("time_limit", -1.0)):
        c = capi.ServerConfig.from_buffer_copy(cfg)
        setattr(c, field, value)
        assert L.lbm_server_create(ctypes.byref(c), ctypes.byref(srv)) == capi.ERR_INVALID
    assert L.lbm_batch_slot_bytes(capi.F32, 0, 8) == -1
    # two population buffers, link words, flags padded to 8 bytes and the 8-byte fluid count
    assert L.lbm_batch_slot_bytes(capi.F16S, 64, 64) == 2 * 9 * 64 * 64 * 2 + 64 * 64 * 2 + 64 * 64 + 8
    assert L.lbm_batch_slot_bytes(capi.F32, 33, 3) == 2 * 9 * 64 * 3 * 4 + 64 * 3 * 2 + 104 + 8


def test_checkpoint_header_errors_without_a_gpu(tmp_path):
    """lbm_checkpoint_desc reads only the file: a missing file and a file that is not a checkpoint
    are rejected with LBM_ERR_INVALID."""
    import ctypes
    from latticeboltzmanncuda_gb300 import capi
    d = capi.Desc()
    assert capi.lib().lbm_checkpoint_desc(str(tmp_path / "missing.lbm").encode(), ctypes.byref(d)) == capi.ERR_INVALID
    junk = tmp_path / "junk.lbm"
    junk.write_bytes(b"not a checkpoint" * 20)
    assert capi.lib().lbm_checkpoint_desc(str(junk).encode(), ctypes.byref(d)) == capi.ERR_INVALID
    assert "not a checkpoint" in capi.last_thread_error()
