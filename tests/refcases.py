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


def icosphere(level=3, r=1.0, c=(0.0, 0.0, 0.0)):
    """Closed triangle mesh of a sphere: the icosahedron with every face split in four `level` times,
    vertices pushed onto the sphere.  Returns (vertices, faces)."""
    t = (1 + 5 ** 0.5) / 2
    v = [(-1, t, 0), (1, t, 0), (-1, -t, 0), (1, -t, 0), (0, -1, t), (0, 1, t), (0, -1, -t), (0, 1, -t),
         (t, 0, -1), (t, 0, 1), (-t, 0, -1), (-t, 0, 1)]
    v = [np.array(p, float) / np.linalg.norm(p) for p in v]
    f = [(0, 11, 5), (0, 5, 1), (0, 1, 7), (0, 7, 10), (0, 10, 11), (1, 5, 9), (5, 11, 4), (11, 10, 2), (10, 7, 6),
         (7, 1, 8), (3, 9, 4), (3, 4, 2), (3, 2, 6), (3, 6, 8), (3, 8, 9), (4, 9, 5), (2, 4, 11), (6, 2, 10),
         (8, 6, 7), (9, 8, 1)]
    for _ in range(level):
        cache, nf = {}, []

        def mid(a, b):
            k = (min(a, b), max(a, b))
            if k not in cache:
                p = v[a] + v[b]
                v.append(p / np.linalg.norm(p))
                cache[k] = len(v) - 1
            return cache[k]
        for a, b, cc in f:
            ab, bc, ca = mid(a, b), mid(b, cc), mid(cc, a)
            nf += [(a, ab, ca), (b, bc, ab), (cc, ca, bc), (ab, bc, ca)]
        f = nf
    return np.array(v) * r + np.array(c), f
