"""CPU replay of the D2Q9 kernels' address arithmetic for every thread of every launch shape the
library can use, over many domain sizes: the vectorised step (csrc/d2q9_vec.cuh, single-domain
grids and batch tiles) and the bulk-copy pipeline (csrc/d2q9_bulk.cuh: copy ranges, alignment,
shared-memory indexes, and its slot protocol under random interleavings).  Every population offset
must lie in [0, 9 * plane) and every link-word offset in [0, plane).  The kernels have no
device-side bounds checks, so this replay is where their indexing is checked; keep it in step
with the kernels."""
import itertools
import os

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
    # stores (fluid cells), only for vectors that start inside the row
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


# ------------------------------------------------------------------ bulk-copy pipeline
# csrc/d2q9_bulk.cuh: strips of BW = 512 cells, BV = 4 or 2 cells per consumer lane (NC = 4 or 8
# consumer warps); a slot holds the nine plane segments one output row pulls (BSEG = BW + 16
# elements each, x0 - 8 .. x0 + BW + 8), BW link words and 8 elements of wrapped columns.
BW = 512
NC = BW // (32 * 4)
BSEG = BW + 16
BLINKS, BWRAP, BSLOT = 9 * BSEG, 9 * BSEG + BW, 9 * BSEG + BW + 8
CY = [0, 0, 1, 0, -1, 1, 1, -1, -1]  # c_y of the populations: plane q is pulled from row y - c_y(q)


def bulk_tasks(nx, ny, reverse):
    """(x0, y) of every task in the order blocks take them (task_of)."""
    pitch = (nx + 31) // 32 * 32
    nstrips = (pitch + BW - 1) // BW
    ntasks = nstrips * ny
    for i in range(ntasks):
        j = ntasks - 1 - i if reverse else i
        y, strip = divmod(j, nstrips)
        yield strip * BW, y


def bulk_check(nx, ny, periodic, reverse, BV):
    pitch = (nx + 31) // 32 * 32
    plane = pitch * ny
    for K in (4, 6):  # slot bases and the barriers after the ring keep 16- and 8-byte alignment
        assert all((s * BSLOT * 2) % 16 == 0 for s in range(K + 1))
    assert (BSEG * 2) % 16 == 0 and (BLINKS * 2) % 16 == 0 and BWRAP + 6 <= BSLOT
    t = np.arange(BW // BV)
    lx = 8 + BV * t
    # consumer reads inside one plane row of a slot: lx .. lx+3, lane 0 lx-1, lane 31 lx+4
    assert lx.min() - 1 >= 0 and lx.max() + BV < BSEG and (BV * t + BV - 1).max() < BW
    for x0, y in bulk_tasks(nx, ny, reverse):
        assert x0 < pitch and x0 % 8 == 0
        gx0, gx1, lx1 = max(x0 - 8, 0), min(x0 + BW + 8, pitch), min(x0 + BW, pitch)
        n, nl = gx1 - gx0, lx1 - x0
        assert n > 0 and nl > 0 and (2 * n) % 16 == 0 and (2 * nl) % 16 == 0
        dst = gx0 - (x0 - 8)
        assert dst >= 0 and dst + n <= BSEG and (2 * dst) % 16 == 0
        for q in range(9):
            row = y - CY[q]
            if row < 0 or row >= ny:
                if not periodic & 2:
                    continue  # not copied
                row %= ny
            g = q * plane + row * pitch + gx0
            assert (2 * g) % 16 == 0 and g >= 0 and g + n <= 9 * plane
        gl = y * pitch + x0
        assert (2 * gl) % 16 == 0 and gl + nl <= plane
        ym = y - 1 if y > 0 else (ny - 1 if periodic & 2 else 0)
        yp = y + 1 if y < ny - 1 else (0 if periodic & 2 else ny - 1)
        if periodic & 1:  # lane 1: wrapped columns
            for r in (y, ym, yp):
                if x0 == 0:
                    assert 0 <= 8 * plane + r * pitch + nx - 1 < 9 * plane
                if x0 <= nx - 1 < x0 + BW:
                    assert 0 <= 7 * plane + r * pitch < 9 * plane
        xc = x0 + BV * t
        # own populations from global memory at the clamped vector
        xa = np.minimum(xc, pitch - BV)
        own = np.arange(9)[:, None] * plane + y * pitch + xa[None, :]
        assert own.min() >= 0 and (own + BV - 1).max() < 9 * plane
        act = xc < nx
        stores = np.arange(9)[:, None] * plane + y * pitch + xc[act][None, :]
        if stores.size:
            assert stores.min() >= 0 and (stores + BV - 1).max() < 9 * plane and (xc[act] + BV - 1).max() < pitch


@pytest.mark.parametrize("nx,ny", SIZES + [(512, 5), (513, 40), (1023, 33), (4096, 17)])
def test_bulk_pipeline_addresses_stay_in_buffers(nx, ny):
    for periodic, reverse, BV in itertools.product(range(4), (0, 1), (2, 4)):
        bulk_check(nx, ny, periodic, reverse, BV)


def test_bulk_tasks_cover_every_cell_once():
    for nx, ny in itertools.product((1, 100, 512, 1000, 4096), (1, 7, 64, 65)):
        pitch = (nx + 31) // 32 * 32
        for reverse in (0, 1):
            seen = np.zeros((ny, pitch), int)
            for x0, y in bulk_tasks(nx, ny, reverse):
                seen[y, x0:min(x0 + BW, pitch)] += 1
            assert (seen == 1).all()


class Barrier:
    """mbarrier phase semantics: a phase completes when its pending arrivals (and bytes) reach 0;
    try_wait.parity(P) succeeds when the current phase's parity differs from P.  Waiting for phase
    m is only unambiguous while at most m + 1 phases have completed."""

    def __init__(self, count):
        self.count, self.pending, self.tx, self.done = count, count, 0, 0

    def arrive(self, tx=0):
        self.pending -= 1
        self.tx += tx
        self._maybe_complete()

    def land(self, nbytes):
        self.tx -= nbytes
        self._maybe_complete()

    def _maybe_complete(self):
        if self.pending == 0 and self.tx == 0:
            self.done += 1
            self.pending = self.count

    def waited(self, m):
        assert self.done <= m + 1, "parity wait would be ambiguous"
        return self.done > m


def simulate_bulk_protocol(ntasks, K, wrap_lane, seed, consumers=NC, arrivals=NC):
    """pipeline(): producer lane 0 (copies, landing at random later times), optionally lane 1 (the
    wrapped columns) and `consumers` consumer warps, each empty barrier expecting `arrivals` (both
    the number of consumer warps in the kernel), under a random interleaving."""
    rng = np.random.default_rng(seed)
    full = [Barrier(2 if wrap_lane else 1) for _ in range(K)]
    empty = [Barrier(arrivals) for _ in range(K)]
    released = [set() for _ in range(consumers)]
    written = {}  # (slot, lane) -> position last written by that producer lane
    ppos = [0, 0 if wrap_lane else ntasks]
    in_flight = []
    cpos = [0] * consumers

    def producer_step(ln):
        p = ppos[ln]
        if p >= ntasks:
            return False
        s = p % K
        if p >= K and not empty[s].waited(p // K - 1):
            return False
        if (s, ln) in written:  # every consumer has released what this lane wrote there before
            assert all(written[(s, ln)] in r for r in released), "slot refilled while live"
        written[(s, ln)] = p
        if ln == 0:
            full[s].arrive(tx=1)
            in_flight.append(s)
        else:
            full[s].arrive()
        ppos[ln] += 1
        return True

    def land_step():
        if not in_flight:
            return False
        full[in_flight.pop(int(rng.integers(len(in_flight))))].land(1)
        return True

    def consumer_step(c):
        p = cpos[c]
        if p >= ntasks:
            return False
        s = p % K
        if not full[s].waited(p // K):
            return False
        assert written.get((s, 0)) == p and (not wrap_lane or written.get((s, 1)) == p), "read a stale slot"
        released[c].add(p)
        empty[s].arrive()
        cpos[c] += 1
        return True

    actors = [lambda: producer_step(0), lambda: producer_step(1), land_step]
    actors += [lambda c=c: consumer_step(c) for c in range(consumers)]
    while True:
        if not any(actors[a]() for a in rng.permutation(len(actors))):
            break
    assert ppos[0] == ntasks and not in_flight, "producer stalled"
    assert all(p == ntasks for p in cpos), "a consumer stalled"


@pytest.mark.parametrize("K", [2, 4, 6])
@pytest.mark.parametrize("consumers", [4, 8])
def test_bulk_slot_protocol_never_deadlocks_or_overwrites(K, consumers):
    for seed in range(30):
        simulate_bulk_protocol(int(np.random.default_rng(seed).integers(1, 40)), K, seed % 2 == 1, seed,
                               consumers=consumers, arrivals=consumers)


def test_bulk_protocol_simulation_catches_a_missing_release():
    """A consumer warp that never released its slots would stall the producer: the simulation
    reports it."""
    with pytest.raises(AssertionError):
        simulate_bulk_protocol(20, 4, False, 0, consumers=NC - 1)


# ------------------------------------------------------------------ batch parameter-block path
# csrc/batch.cu: slots are one allocation each (buffer A, buffer B: 9 planes of pitch x ny elements
# each; then pitch x ny uint16 link words; then flags and the fluid count).  16-bit storage: flat
# tiles -- tile j of a slot covers the tx * ty * V consecutive cells from j * tx * ty * V of the slot's
# padded cell array, thread k of the block the vector at j * tx * ty * V + k * V (d2q9_vec.cuh:
# step_vec_flat).  FP32: row-band tiles -- (slot, band of ty rows, column chunk of tx * V cells).  A
# block finds its slot by a binary search over the slots' first tiles.


def batch_tiles(shapes, V, tx, ty):
    """Every tile of a launch as (slot, tile within the slot), and the slots' first tiles (rebuild())."""
    tiles, start = [], []
    per_tile = tx * ty * V
    for k, (nx, ny) in enumerate(shapes):
        pitch = (nx + 31) // 32 * 32
        start.append(len(tiles))
        tiles += [(k, j) for j in range((pitch * ny + per_tile - 1) // per_tile)]
    return tiles, start


PREFETCH_CELLS = 32768  # batch.cu: PREFETCH_CELLS
CY = [0, 0, 1, 0, -1, 1, 1, -1, -1]  # c_y of the D2Q9 populations


def test_prefetch_distance_matches_the_kernel_source():
    src = os.path.join(os.path.dirname(os.path.dirname(os.path.abspath(__file__))),
                       "latticeboltzmanncuda_gb300", "csrc", "batch.cu")
    with open(src) as fh:
        assert f"constexpr int PREFETCH_CELLS = {PREFETCH_CELLS};" in fh.read()


def search_tile(start, t):
    """batch_tile_p's binary search for tile t: (slot, tile within the slot)."""
    lo, hi = 0, len(start) - 1
    while lo < hi:
        mid = (lo + hi + 1) >> 1
        if start[mid] <= t:
            lo = mid
        else:
            hi = mid - 1
    return lo, t - start[lo]


def pitch_division(pitch):
    """(multiplier, shift) of batch_tile_p's division by the pitch, as rebuild() computes them."""
    l = 0
    while (1 << l) < pitch:
        l += 1
    return ((1 << 32) * ((1 << l) - pitch) // pitch + 1) & 0xFFFFFFFF, l - 1


def divide(i, magic, shift):
    """batch_tile_p's multiply-high division (i: int or uint64 array below 2^31)"""
    th = (np.uint64(magic) * np.asarray(i, np.uint64)) >> np.uint64(32)
    return (th + ((np.asarray(i, np.uint64) - th) >> np.uint64(1))) >> np.uint64(shift)


def flat_thread_offsets(nx, ny, pitch, V, x0, y, lane, periodic, active):
    """(population offsets, link offsets) one lane of step_vec_flat touches (element indices)."""
    plane = pitch * ny
    ym = np.where(y - 1 < 0, ny - 1 if periodic & 2 else 0, y - 1)
    yp = np.where(y + 1 >= ny, 0 if periodic & 2 else ny - 1, y + 1)
    r0, rm, rp = y * pitch, ym * pitch, yp * pitch
    pop, lnk = [], []
    for q, r in {0: r0, 2: rm, 4: rp, 1: r0, 5: rm, 8: rp, 3: r0, 6: rm, 7: rp}.items():
        for k in range(V):
            pop.append(q * plane + r + x0 + k)
            pop.append(q * plane + r0 + x0 + k)  # own populations (bounce-back)
    for k in range(V):
        lnk.append(r0 + x0 + k)
    left = (lane == 0) | (x0 == 0)
    right = (lane == 31) | (x0 + V == pitch)
    xm = np.where(x0 - 1 < 0, nx - 1 if periodic & 1 else 0, x0 - 1)
    xq = np.minimum(x0 + V, pitch - 1)
    for q, r in ((1, r0), (5, rm), (8, rp)):
        pop.append(np.where(left, q * plane + r + xm, 0))
    for q, r in ((3, r0), (6, rm), (7, rp)):
        pop.append(np.where(right, q * plane + r + xq, 0))
    kl = nx - 1 - x0
    mp = bool(periodic & 1) & (kl >= 0) & (kl < V)
    for q, r in ((3, r0), (6, rm), (7, rp)):
        pop.append(np.where(mp, q * plane + r, 0))
    st = active & (x0 < nx)
    for q in range(9):
        for k in range(V):
            pop.append(np.where(st, q * plane + r0 + x0 + k, 0))
    return np.stack(pop), np.stack(lnk)


def flat_lanes(nx, ny, V, tx, ty, j):
    """x0, y, lane, active of the lanes of tile j (an int, or an array of tiles: their lanes one tile
    after another) that run (warps past the slot's end return)."""
    pitch = (nx + 31) // 32 * 32
    plane = pitch * ny
    magic, shift = pitch_division(pitch)
    k = np.tile(np.arange(tx * ty), np.size(j))
    first = np.repeat(np.asarray(j).reshape(-1) * tx * ty * V, tx * ty)
    runs = first + (k & ~31) * V < plane
    k, first = k[runs], first[runs]
    i = first + k * V
    active = i < plane
    i = np.where(active, i, plane - V)
    y = divide(i, magic, shift).astype(np.int64)
    assert np.array_equal(y, i // pitch)
    return i - y * pitch, y, k % 32, active


@pytest.mark.parametrize("seed", range(3))
def test_batch_parameter_path_tiles_and_addresses(seed):
    rng = np.random.default_rng(seed)
    n = int(rng.integers(1, 30))
    shapes = [(int(rng.integers(1, 700)), int(rng.integers(1, 300))) for _ in range(n)]
    shapes += [(1, 1), (32, 1), (33, 3), (64, 5)]
    for elem, V, tx, ty in ((2, 4, 32, 4), (2, 8, 32, 2), (2, 2, 64, 1), (2, 4, 32, 1), (2, 8, 256, 1)):
        tiles, start = batch_tiles(shapes, V, tx, ty)
        # the binary search finds every tile's slot and index within the slot
        for t, rec in enumerate(tiles):
            assert search_tile(start, t) == rec
        for k, (nx, ny) in enumerate(shapes):
            pitch = (nx + 31) // 32 * 32
            plane = pitch * ny
            pop = 9 * plane * elem
            alloc = 2 * pop + plane * 2 + ((nx * ny + 7) // 8 * 8 + 8)
            seen = np.zeros((ny, pitch), int)
            js = np.array([j for (kk, j) in tiles if kk == k])
            for j in (js,):
                x0, y, lane, active = flat_lanes(nx, ny, V, tx, ty, j)
                assert (x0 % V == 0).all() and (x0 >= 0).all() and (x0 + V <= pitch).all()
                for periodic in range(4):
                    offs, lnk = flat_thread_offsets(nx, ny, pitch, V, x0, y, lane, periodic, active)
                    assert offs.min() >= 0 and offs.max() < 9 * plane, (nx, ny, V, tx, ty, periodic)
                    assert lnk.min() >= 0 and lnk.max() < plane
                # byte offsets from the slot's base: both buffers and the link words lie in the allocation
                assert (9 * plane + 9 * plane) * elem == 2 * pop
                assert 2 * pop + (int(lnk.max()) + 1) * 2 <= alloc
                st = active & (x0 < nx)
                for e in range(V):
                    np.add.at(seen, (y[st], x0[st] + e), 1)
            # the L2 prefetch of the tile PREFETCH_CELLS further along (16-bit flat tiles) stays in
            # the slot's planes, 16-byte aligned
            per = tx * ty * V
            for j in range(len(js)):
                for d in (1, -1):
                    tf = j + d * (PREFETCH_CELLS // per)
                    if plane < per or tf < 0 or tf * per >= plane:
                        continue
                    first = min(tf * per, plane - per)
                    for q in range(9):
                        o = max(0, min(first - CY[q] * pitch, plane - per))
                        assert 0 <= o and o + per <= plane and (o * elem) % 16 == 0 and (per * elem) % 16 == 0
                    assert first + per <= plane and (first * 2) % 16 == 0
            # every cell of every slot belongs to exactly one storing lane (which skips solid cells)
            assert (seen[:, :nx] == 1).all(), (nx, ny, V, tx, ty)


def test_flat_lane_edges_take_their_own_neighbours():
    """A lane that starts a padded row (or is lane 0) loads its x - 1 neighbours, a lane that ends one
    (or is lane 31) its x + V neighbours; every other lane's neighbours are the adjacent lanes' own
    vectors in the same row, so the shuffles never carry a value across a row boundary."""
    for nx, ny, V, tx, ty in ((40, 9, 4, 32, 4), (31, 17, 8, 32, 2), (100, 3, 2, 64, 1), (1, 70, 4, 32, 1)):
        pitch = (nx + 31) // 32 * 32
        for j in range((pitch * ny + tx * ty * V - 1) // (tx * ty * V)):
            x0, y, lane, active = flat_lanes(nx, ny, V, tx, ty, j)
            left = (lane == 0) | (x0 == 0)
            right = (lane == 31) | (x0 + V == pitch)
            for a in range(len(x0)):
                if not left[a] and active[a]:  # lanes past the slot's end store nothing
                    assert lane[a - 1] == lane[a] - 1 and y[a - 1] == y[a] and x0[a - 1] == x0[a] - V
                if not right[a] and active[a]:
                    assert lane[a + 1] == lane[a] + 1 and y[a + 1] == y[a] and x0[a + 1] == x0[a] + V


def band_tiles(shapes, V, tx, ty):
    """FP32 row-band tiles of rebuild(): (slot, band, xchunk) per tile, and the slots' first tiles."""
    tiles, start = [], []
    for k, (nx, ny) in enumerate(shapes):
        pitch = (nx + 31) // 32 * 32
        chunks = (pitch // V + tx - 1) // tx
        start.append(len(tiles))
        for band in range((ny + ty - 1) // ty):
            for xc in range(chunks):
                tiles.append((k, band, xc))
    return tiles, start


def search_band_tile(start, t, chunks):
    """batch_tile_p's binary search and division for a row-band tile t."""
    lo, hi = 0, len(start) - 1
    while lo < hi:
        mid = (lo + hi + 1) >> 1
        if start[mid] <= t:
            lo = mid
        else:
            hi = mid - 1
    i = t - start[lo]
    return lo, i // chunks[lo], i - (i // chunks[lo]) * chunks[lo]


@pytest.mark.parametrize("seed", range(3))
def test_batch_parameter_path_row_bands_fp32(seed):
    rng = np.random.default_rng(seed)
    n = int(rng.integers(1, 30))
    shapes = [(int(rng.integers(1, 700)), int(rng.integers(1, 300))) for _ in range(n)]
    for elem, V, tx, ty in ((4, 4, 32, 2), (4, 2, 128, 2), (4, 4, 64, 1), (4, 2, 32, 8)):
        tiles, start = band_tiles(shapes, V, tx, ty)
        chunks = [((nx + 31) // 32 * 32 // V + tx - 1) // tx for nx, _ in shapes]
        # the binary search finds every tile's slot, band and column chunk
        for t, rec in enumerate(tiles):
            assert search_band_tile(start, t, chunks) == rec
        # every cell of every slot is covered by exactly one (tile, thread row, lane, element)
        for k, (nx, ny) in enumerate(shapes):
            pitch = (nx + 31) // 32 * 32
            plane = pitch * ny
            pop = 9 * plane * elem
            alloc = 2 * pop + plane * 2 + ((nx * ny + 7) // 8 * 8 + 8)
            seen = np.zeros((ny, pitch), int)
            for (kk, band, xc) in (r for r in tiles if r[0] == k):
                for ti in range(ty):
                    y = band * ty + ti
                    if y >= ny:
                        continue
                    x0 = (xc * tx + np.arange(tx)) * V
                    xa = np.minimum(x0, pitch - V)
                    for cur in (0, 1):
                        src = cur * 9 * plane  # elements from the base
                        dst = (cur ^ 1) * 9 * plane
                        for base in (src, dst):
                            offs = base + 8 * plane + y * pitch + xa + V - 1  # the highest plane and element
                            assert offs.max() * elem < pop * (2 if base else 1)
                    links = 18 * plane * elem  # byte offset of the link words
                    assert links == 2 * pop and links + (y * pitch + xa.max() + V) * 2 <= alloc
                    act = x0 < nx
                    for x in x0[act]:
                        seen[y, x:x + V] += 1
            assert (seen[:, :nx] == 1).all()


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


D3_PREFETCH_BLOCKS = 128  # d3q27.cu: D3_PREFETCH_BLOCKS
KD27 = None


def _kd27():
    """the D3Q27 direction table of d3q27.cu's kd(j, a), read from the source"""
    global KD27
    if KD27 is None:
        import re
        src = os.path.join(os.path.dirname(os.path.dirname(os.path.abspath(__file__))),
                           "latticeboltzmanncuda_gb300", "csrc", "d3q27.cu")
        with open(src) as fh:
            text = fh.read()
        assert f"constexpr int D3_PREFETCH_BLOCKS = {D3_PREFETCH_BLOCKS};" in text
        body = text[text.index("constexpr int kd(int j, int a)"):]
        body = body[body.index("{", body.index("t[27][3]")):body.index("};")]
        vals = [int(v) for v in re.findall(r"-?\d+", body)]
        KD27 = np.array(vals[:81]).reshape(27, 3)
    return KD27


@pytest.mark.parametrize("dims", [(128, 128, 128), (5, 7, 3), (33, 17, 50), (1, 1, 130), (64, 3, 129)])
def test_d3q27_prefetch_stays_in_the_population_buffer(dims):
    """fused_kernel<FP32>'s L2 prefetch: for every block, each of the 27 segments lies inside the
    27-plane buffer and starts on a 16-byte boundary."""
    X, Y, Z = dims
    n = X * Y * Z
    kd = _kd27()
    threads = 128
    length = threads + 4
    total = 27 * n
    for b in range((n + threads - 1) // threads):
        first = (b + D3_PREFETCH_BLOCKS) * threads
        if first + threads > n or total < length:
            continue
        for j in range(27):
            off = kd[j, 2] + Z * (kd[j, 1] + Y * kd[j, 0])
            e = j * n + first - off
            e = 0 if e < 0 else (total - length if e > total - length else e)
            e &= ~3
            assert 0 <= e and e + length <= total and (e * 4) % 16 == 0


CX = [0, 1, 0, -1, 0, 1, -1, -1, 1]  # c_x of the D2Q9 populations


@pytest.mark.parametrize("elem,tx,ty", [(4, 64, 8), (4, 64, 16), (4, 128, 8), (2, 64, 8), (2, 64, 16), (2, 128, 8),
                                         (4, 64, 4), (2, 64, 4)])
def test_two_step_tile_indexing(elem, tx, ty):
    """d2q9_tile2.cuh: every global load and store lies in the planes, every shared-memory index in
    its tile, for domains smaller and larger than a tile, periodic or not; the shared memory fits."""
    iw, ih, mw, mh = tx + 4, ty + 4, tx + 2, ty + 2
    n_in, n_mid = iw * ih, mw * mh
    smem = 9 * n_in * elem + 9 * n_mid * elem + n_mid * 2
    assert smem <= 227 * 1024
    # the persistent form: two input buffers with the link words of the loaded tile, then mid
    buf = (9 * n_in * elem + n_in * 2 + 15) // 16 * 16
    assert 2 * buf + 9 * n_mid * elem <= 227 * 1024 and (9 * n_in * elem) % 16 == 0
    rng = np.random.default_rng(tx * 100 + ty + elem)
    shapes = [(1, 1), (5, 3), (tx, ty), (tx + 1, ty + 3), (3 * tx + 7, 2 * ty + 1)] + \
             [(int(rng.integers(1, 400)), int(rng.integers(1, 90))) for _ in range(4)]
    for nx, ny in shapes:
        pitch = (nx + 31) // 32 * 32
        plane = pitch * ny
        for periodic in range(4):
            px, py = bool(periodic & 1), bool(periodic & 2)

            def wc(g, n, per):
                inside = (g >= 0) & (g < n)
                w = np.where(per, np.mod(g, n), np.clip(g, 0, n - 1))
                return np.where(inside, g, w), inside | per

            for bx in range((nx + tx - 1) // tx):
                for by in range((ny + ty - 1) // ty):
                    x0, y0 = bx * tx, by * ty
                    # loads of the two-cell halo tile
                    j, i = np.divmod(np.arange(n_in), iw)
                    gx, _ = wc(x0 - 2 + i, nx, px)
                    gy, _ = wc(y0 - 2 + j, ny, py)
                    g = gy * pitch + gx
                    assert g.min() >= 0 and g.max() < plane
                    # link words of the mid tile
                    j, i = np.divmod(np.arange(n_mid), mw)
                    gx, inx = wc(x0 - 1 + i, nx, px)
                    gy, iny = wc(y0 - 1 + j, ny, py)
                    assert (gy * pitch + gx).min() >= 0 and (gy * pitch + gx).max() < plane
                    # first step: pulls from the in tile around (i + 1, j + 1)
                    c = (j + 1) * iw + (i + 1)
                    for q in range(9):
                        s = c - CY[q] * iw - CX[q]
                        assert s.min() >= 0 and s.max() < n_in
                    # second step: pulls from the mid tile around (i + 1, j + 1), stores in the planes
                    j, i = np.divmod(np.arange(tx * ty), tx)
                    keep = (x0 + i < nx) & (y0 + j < ny)
                    m = (j + 1) * mw + (i + 1)
                    assert m.max() < n_mid
                    for q in range(9):
                        s = m - CY[q] * mw - CX[q]
                        assert s.min() >= 0 and s.max() < n_mid
                    gs = (y0 + j[keep]) * pitch + x0 + i[keep]
                    if gs.size:
                        assert gs.min() >= 0 and gs.max() < plane
