"""Set-ups of the reference's known-answer tests (test/CalculationsTest.cpp), shared by the oracle
golden tests and the GPU parity tests.  Each builder returns numpy inputs in the cell-major
layout f[cell, 27], cell = z + Z*(y + Y*x) (the reference host index, Lattice.cpp:254)."""
from __future__ import annotations

import numpy as np

REFL_DTYPE = np.dtype([("dirs", np.int32, (14,)), ("w", np.float32, (81,))])
INTERNAL, REFLECTED, SOURCE = 1, 2, 4


def cell(dims, x, y, z):
    X, Y, Z = dims
    return z + Z * (y + Y * x)


def pack_dir(rec, slot, d):
    """5-bit direction packing of Lattice.cpp:450-463."""
    w = np.uint32(rec["dirs"][slot // 6].view(np.uint32))
    sh = 5 * (slot % 6)
    w = (w & ~np.uint32(31 << sh)) | np.uint32((d & 31) << sh)
    rec["dirs"][slot // 6] = np.int32(w.view(np.int32))


def cube_angled_table(golden):
    """Reflection record of cell (1,1,1) of the 3x3x3 / spacing 0.5 cube_angled lattice, with the
    three slots the reference pins (CoordinatesTest.cpp:223-228): population 1 -> slots 3, 4, 5."""
    from conftest import known
    tabs = np.zeros(1, dtype=REFL_DTYPE)
    for slot, line_w, line_d in ((3, 223, 226), (4, 224, 227), (5, 225, 228)):
        w = known(golden, "CoordinatesTest.TestReflection", line_w)["value"]
        d = int(known(golden, "CoordinatesTest.TestReflection", line_d)["value"])
        tabs[0]["w"][slot] = w
        pack_dir(tabs[0], slot, d)
    return tabs


def reflections_case(golden):
    """CalculationsTest.cpp:107-146 / 148-197: f1 = 1 at (1,1,1), the only internal cell of
    cube_angled at spacing 0.5 on 3x3x3; everything else zero."""
    dims = (3, 3, 3)
    n = 27
    f = np.zeros((n, 27), dtype=np.float32)
    c = cell(dims, 1, 1, 1)
    f[c, 1] = 1.0
    flags = np.zeros(n, dtype=np.uint8)
    flags[c] = INTERNAL | REFLECTED
    tab_idx = np.full(n, -1, dtype=np.int32)
    tab_idx[c] = 0
    return dims, f, flags, tab_idx, cube_angled_table(golden)
