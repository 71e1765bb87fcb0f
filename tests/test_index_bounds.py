"""CPU replay of the vectorised D2Q9 step's address arithmetic (csrc/d2q9_vec.cuh, step_vec) for
every thread of every launch shape the library can use, single-domain grids and batch tiles,
over many domain sizes: every population offset must lie in [0, 9 * plane) and every link-word
offset in [0, plane).  The kernel has no device-side bounds checks, so this replay is where its
indexing is checked; keep it in step with step_vec."""
import itertools

import numpy as np
import pytest


def thread_offsets(nx, ny, pitch, V, x0, y, lane, periodic):
    """(population offsets, link offsets) one thread of step_vec touches, as element indices."""
    plane = pitch * ny
    xa = np.minimum(x0, pitch - V)
    ym = y - 1
    yp = y + 1
    ym = np.where(ym < 0, ny - 1 if periodic & 2 else 0, ym)
    yp = np.where(yp >= ny, 0 if periodic & 2 else ny - 1, yp)
    r0, rm, rp = y * pitch, ym * pitch, yp * pitch
    pop, lnk = [], []
    rows = {0: r0, 2: rm, 4: rp, 1: r0, 5: rm, 8: rp, 3: r0, 6: rm, 7: rp}
    for q, r in rows.items():
        for k in range(V):
            pop.append(q * plane + r + xa + k)
    for k in range(V):
        lnk.append(r0 + xa + k)
    # lane 0: left neighbour from the clamped xa, wrapped or clamped at x = 0
    xm = xa - 1
    xm = np.where(xm < 0, nx - 1 if periodic & 1 else 0, xm)
    m0 = lane == 0
    for q, r in ((1, r0), (5, rm), (8, rp)):
        pop.append(np.where(m0, q * plane + r + xm, 0))
    # lane 31: right neighbour, clamped to the row
    xq = np.minimum(x0 + V, pitch - 1)
    m31 = lane == 31
    for q, r in ((3, r0), (6, rm), (7, rp)):
        pop.append(np.where(m31, q * plane + r + xq, 0))
    # periodic patch of the last column from x = 0
    kl = nx - 1 - x0
    mp = bool(periodic & 1) & (kl >= 0) & (kl < V)
    for q, r in ((3, r0), (6, rm), (7, rp)):
        pop.append(np.where(mp, q * plane + r, 0))
    # own populations for bounce-back (any q), at xa
    for q in range(9):
        for k in range(V):
            pop.append(q * plane + r0 + xa + k)
    # solid copies and stores, only for vectors that start inside the row
    act = x0 < nx
    for q in range(9):
        for k in range(V):
            pop.append(np.where(act, q * plane + r0 + x0 + k, 0))
    return np.stack(pop), np.stack(lnk), plane


def check(nx, ny, V, tx, ty, periodic, batch):
    pitch = (nx + 31) // 32 * 32
    per_row = pitch // V
    chunks = (per_row + tx - 1) // tx
    xs, ys, lanes = [], [], []
    for yb in range(0, ny if batch else (ny + ty - 1) // ty * ty, ty):
        for xc in range(chunks):
            for ti in range(ty):
                y = yb + ti
                if y >= ny:
                    continue  # the kernel returns before any access
                t = np.arange(tx)
                xs.append((xc * tx + t) * V)
                ys.append(np.full(tx, y))
                lanes.append(t % 32)
    x0, y, lane = np.concatenate(xs), np.concatenate(ys), np.concatenate(lanes)
    pop, lnk, plane = thread_offsets(nx, ny, pitch, V, x0, y, lane, periodic)
    assert pop.min() >= 0 and pop.max() < 9 * plane, (nx, ny, V, tx, ty, periodic, pop.max() - 9 * plane)
    assert lnk.min() >= 0 and lnk.max() < plane, (nx, ny, V, tx, ty, periodic)


SIZES = [(1, 1), (5, 3), (31, 7), (33, 2), (64, 64), (150, 41), (203, 77), (1000, 9), (4096, 3)]
SHAPES = [(V, tx, ty) for V in (2, 4, 8) for tx in (32, 64, 128, 256) for ty in (1, 2, 4, 8) if tx * ty <= 256]


@pytest.mark.parametrize("nx,ny", SIZES)
def test_vector_step_addresses_stay_in_buffers(nx, ny):
    for (V, tx, ty), periodic, batch in itertools.product(SHAPES, range(4), (False, True)):
        check(nx, ny, V, tx, ty, periodic, batch)


def test_replay_catches_an_unclamped_left_neighbour():
    """The replay would have flagged lane 0's left neighbour taken from x0 instead of xa: a warp
    wholly beyond a narrow row reads past the last plane."""
    nx, ny, V, tx = 150, 41, 8, 128
    pitch = (nx + 31) // 32 * 32
    plane = pitch * ny
    x0 = np.array([(3 * 32) * V])  # lane 0 of the fourth warp, beyond the 160-wide row
    bad = 8 * plane + (ny - 1) * pitch + (x0 - 1)
    assert bad.max() >= 9 * plane


# ------------------------------------------------------------------ shared-memory row sweep
# csrc/d2q9_stage.cuh: 128 threads x 4 cells = strips of W = 512, plane rows of SEG = W + 16
# elements staged as 16-byte (8-element) chunks, link words after the nine planes of a slot.
THREADS, CPT = 128, 4
W = THREADS * CPT
SEG = W + 16
CHUNKS, LCHUNKS = SEG // 8, W // 8
LINKS, SLOT = 9 * SEG, 9 * SEG + W


def stage_offsets(nx, ny, rows, periodic, nslot):
    """Every global element offset and shared-memory index the row sweep touches, over all blocks."""
    pitch = (nx + 31) // 32 * 32
    plane = pitch * ny
    gread, lread, gwrite, smem = [], [], [], []
    nbx, nby = (nx + W - 1) // W, (ny + rows - 1) // rows
    t = np.arange(THREADS)
    for bx in range(nbx):
        x0 = bx * W
        for by in range(nby):
            ya = by * rows
            yb = min(ya + rows, ny)
            for p in range(yb - ya + 2):  # copies of rows ya-1 .. yb
                row = ya - 1 + p
                if row < 0 or row >= ny:
                    if not periodic & 2:
                        continue
                    row = row + ny if row < 0 else row - ny
                base = (p % nslot) * SLOT
                tp = t[t < CHUNKS]
                gx = x0 - 8 + 8 * tp
                ok = (gx >= 0) & (gx + 8 <= pitch)
                for q in range(9):
                    g = q * plane + row * pitch + gx[ok]
                    gread += [g, g + 7]
                    smem += [base + q * SEG + 8 * tp[ok], base + q * SEG + 8 * tp[ok] + 7]
                lt = t - (THREADS - LCHUNKS)
                lt = lt[lt >= 0]
                gl = x0 + 8 * lt
                okl = gl + 8 <= pitch
                lread += [row * pitch + gl[okl], row * pitch + gl[okl] + 7]
                smem += [base + LINKS + 8 * lt[okl], base + LINKS + 8 * lt[okl] + 7]
            xa = x0 + CPT * t
            act = xa < nx
            lx = 8 + CPT * t[act]
            for k, y in enumerate(range(ya, yb)):
                c = y * pitch + xa[act]
                for q in range(9):
                    gwrite += [q * plane + c, q * plane + c + CPT - 1]  # one 8-byte store
                for d in range(3):
                    base = ((k + d) % nslot) * SLOT
                    smem += [base + 8 * SEG + lx - 1, base + 8 * SEG + lx + CPT]  # reads lx-1 .. lx+4 of a plane
                    smem += [base + LINKS + CPT * t[act], base + LINKS + CPT * t[act] + CPT - 1]
                if periodic & 1:
                    ym = y - 1 if y > 0 else (ny - 1 if periodic & 2 else 0)
                    yp = y + 1 if y < ny - 1 else (0 if periodic & 2 else ny - 1)
                    cells = np.concatenate([xa[act] + cc for cc in range(CPT)])
                    for q, r in ((1, y), (5, ym), (8, yp)):
                        gread.append(q * plane + r * pitch + np.full(int((cells == 0).sum()), nx - 1))
                    for q, r in ((3, y), (6, ym), (7, yp)):
                        gread.append(q * plane + r * pitch + np.zeros(int((cells == nx - 1).sum()), int))
    cat = lambda a: np.concatenate(a) if a else np.zeros(0, int)
    return cat(gread), cat(lread), cat(gwrite), cat(smem), plane


@pytest.mark.parametrize("nx,ny", SIZES + [(512, 5), (513, 40), (1023, 33)])
def test_row_sweep_addresses_stay_in_buffers(nx, ny):
    for rows, periodic, nslot in itertools.product((1, 8, 64), range(4), (4, 8)):
        gread, lread, gwrite, smem, plane = stage_offsets(nx, ny, rows, periodic, nslot)
        for a, hi in ((gread, 9 * plane), (lread, plane), (gwrite, 9 * plane), (smem, nslot * SLOT)):
            if a.size:
                assert a.min() >= 0 and a.max() < hi, (nx, ny, rows, periodic, nslot, a.min(), a.max(), hi)


@pytest.mark.parametrize("nslot", [4, 8])
def test_row_sweep_slot_reuse_never_overwrites_a_live_row(nslot):
    """Iteration k reads positions k, k+1, k+2 and refills the slot of position k + nslot - 1,
    which is the slot of position k - 1: no slot is refilled while a live row sits in it; and
    waiting until at most nslot - 4 copy groups are pending leaves positions <= k + 2 landed."""
    for k in range(200):
        live = {(k + d) % nslot for d in range(3)}
        assert (k + nslot - 1) % nslot not in live
        committed = (nslot - 1) + k  # prologue groups + one per earlier iteration
        assert committed - (nslot - 4) >= k + 3


def test_invariant_division_formula():
    """The D3Q27 kernels turn cell indices into (x, y, z) by the multiply-high division of
    csrc/d3q27.cu (FastDiv, Granlund-Montgomery 1994): checked against integer division for every
    divisor up to 2000, powers of two and neighbours, random divisors and numerators up to 2^32-1."""
    import random

    def fastdiv(n, d):
        l = 0
        while l < 32 and (1 << l) < d:
            l += 1
        m = ((1 << 32) * ((1 << l) - d) // d + 1) & 0xFFFFFFFF
        t = (m * n) >> 32
        return (t + ((n - t) >> min(l, 1))) >> max(l - 1, 0)

    rng = random.Random(1)
    divisors = list(range(1, 2000)) + [rng.randrange(1, 2 ** 31) for _ in range(500)]
    divisors += [2 ** k + e for k in range(1, 31) for e in (-1, 0, 1)]
    for d in divisors:
        for n in [0, 1, d - 1, d, d + 1, 2 * d - 1, 2 ** 31 - 1, 2 ** 32 - 1] + [rng.randrange(2 ** 32) for _ in range(50)]:
            assert fastdiv(n, d) == n // d, (n, d)
