"""D2Q9 parity: the CUDA kernels (through the C ABI) against the CPU oracle on the same seeded inputs.

Tolerances (stated per storage type):
  FP64 storage  max |f_gpu - f_oracle| <= 1e-12   (same arithmetic, different evaluation order)
  FP32 storage  max |f_gpu - f_oracle64| <= 1e-5 * max|f|, and velocity field within 1e-4 of max|u|
                relative after the run (FP32 rounding accumulated over the run)
  FP16/BF16-shifted storage on a 48 x 40 lid-driven cavity after 400 steps: relative velocity L2
                within 1e-3 / 1e-2 and max within 2e-3 / 2e-2 (storage precision 2^-11 / 2^-8 of the
                shifted populations; the benchmark-size cases are in test_gpu_configs.py)
"""
import zlib

import numpy as np
import pytest

import latticeboltzmanncuda_gb300 as lbm
import oracle

pytestmark = pytest.mark.gpu


def box(nx, ny, lid=False):
    fl = np.zeros((ny, nx), np.uint8)
    fl[0, :] = 1
    fl[:, 0] = 1
    fl[:, -1] = 1
    fl[-1, :] = 2 if lid else 1
    return fl


def random_state(nx, ny, seed, amp=0.02):
    rng = np.random.default_rng(seed)
    rho = 1 + amp * rng.standard_normal((ny, nx))
    ux = amp * rng.standard_normal((ny, nx))
    uy = amp * rng.standard_normal((ny, nx))
    f = oracle.d2q9_equilibrium(rho, ux, uy)
    f += 1e-3 * rng.standard_normal(f.shape)  # non-equilibrium part
    return f


def gpu_run(flags, f0, tau, steps, periodic=0, force=(0, 0), wall=(0, 0), dtype="f64"):
    _, ny, nx = f0.shape
    with lbm.Lattice(nx, ny, dtype=dtype, tau=tau, periodic=periodic, body_force=(force[0], force[1], 0),
                     wall_velocity=(wall[0], wall[1], 0)) as L:
        L.set_flags(flags)
        L.load_populations(f0)
        L.step(steps)
        f = L.retrieve_populations(np.float64)
        rho, ux, uy = L.moments()
        cons = L.conservation()
    return f, (rho, ux, uy), cons


CASES = {
    # name: (nx, ny, flags builder, periodic, force, wall, tau, steps)
    "closed_box": (37, 23, lambda nx, ny: box(nx, ny), 0, (0, 0), (0, 0), 0.7, 60),
    "cavity_lid": (40, 33, lambda nx, ny: box(nx, ny, lid=True), 0, (0, 0), (0.05, 0), 0.6, 80),
    "channel_force": (64, 20, None, 1, (1e-5, 0), (0, 0), 0.55, 80),
    "periodic_xy_force": (33, 31, lambda nx, ny: np.zeros((ny, nx), np.uint8), 3, (2e-5, -1e-5), (0, 0), 0.9, 50),
    "open_edges": (29, 17, lambda nx, ny: np.zeros((ny, nx), np.uint8), 0, (0, 0), (0, 0), 0.8, 40),
    "periodic_y_moving": (24, 30, None, 2, (0, 0), (0.03, 0.01), 0.65, 50),
    "thin_1xN": (1, 40, lambda nx, ny: np.zeros((ny, nx), np.uint8), 3, (0, 1e-5), (0, 0), 0.75, 30),
    "thin_Nx1": (45, 1, lambda nx, ny: np.zeros((ny, nx), np.uint8), 3, (1e-5, 0), (0, 0), 0.7, 30),
    "single_cell": (1, 1, lambda nx, ny: np.zeros((ny, nx), np.uint8), 3, (2e-5, -1e-5), (0, 0), 0.8, 20),
}


def build_flags(name, nx, ny, builder):
    if builder is not None:
        return builder(nx, ny)
    if name == "channel_force":
        fl, _ = lbm.gen_channel(nx, ny, 2, 2.0, 4.0, 3)
        return fl
    fl = np.zeros((ny, nx), np.uint8)
    fl[:, 0] = 1
    fl[:, -1] = 2
    fl[10:14, 8:12] = 1
    return fl


def f32(*v):
    """lbm_desc carries tau, force and wall velocity as float: the oracle gets the same values."""
    return tuple(float(np.float32(x)) for x in v)


@pytest.mark.parametrize("name", list(CASES))
def test_fp64_gpu_matches_fp64_oracle(name):
    nx, ny, builder, periodic, force, wall, tau, steps = CASES[name]
    (tau,), force, wall = f32(tau), f32(*force), f32(*wall)
    flags = build_flags(name, nx, ny, builder)
    f0 = random_state(nx, ny, zlib.crc32(name.encode()))
    ref = oracle.d2q9_run(f0, flags, tau, steps, periodic=periodic, force=force, wall_velocity=wall)
    got, (rho, ux, uy), cons = gpu_run(flags, f0, tau, steps, periodic, force, wall, "f64")
    fluid = flags == 0
    assert np.max(np.abs(got - ref)[:, fluid]) <= 1e-12
    r_rho, r_ux, r_uy = oracle.d2q9_moments(ref, flags, periodic=periodic, force=force, wall_velocity=wall)
    assert np.max(np.abs(rho - r_rho)[fluid]) < 1e-6
    assert np.max(np.abs(ux - r_ux)[fluid]) < 1e-7
    assert np.max(np.abs(uy - r_uy)[fluid]) < 1e-7
    want = oracle.d2q9_conservation(ref, flags)
    assert np.allclose(cons[:3], want, rtol=1e-12, atol=1e-12)


@pytest.mark.parametrize("name", list(CASES))
def test_fp32_gpu_within_tolerance_of_fp64_oracle(name):
    nx, ny, builder, periodic, force, wall, tau, steps = CASES[name]
    flags = build_flags(name, nx, ny, builder)
    f0 = random_state(nx, ny, zlib.crc32(name.encode()))
    ref = oracle.d2q9_run(f0, flags, tau, steps, periodic=periodic, force=force, wall_velocity=wall)
    got, _, _ = gpu_run(flags, f0, tau, steps, periodic, force, wall, "f32")
    fluid = flags == 0
    err = np.max(np.abs(got - ref)[:, fluid])
    assert err <= 1e-5 * np.max(np.abs(ref)), err


@pytest.mark.parametrize("dtype,tol_l2,tol_max", [("f16s", 1e-3, 2e-3), ("bf16s", 1e-2, 2e-2)])
def test_shifted_half_storage_velocity(dtype, tol_l2, tol_max):
    nx, ny = 48, 40
    flags = box(nx, ny, lid=True)
    f0 = oracle.d2q9_equilibrium(np.ones((ny, nx)), np.zeros((ny, nx)), np.zeros((ny, nx)))
    ref = oracle.d2q9_run(f0, flags, 0.6, 400, wall_velocity=(0.05, 0))
    _, rux, ruy = oracle.d2q9_moments(ref, flags, wall_velocity=(0.05, 0))
    _, (rho, ux, uy), _ = gpu_run(flags, f0, 0.6, 400, 0, (0, 0), (0.05, 0), dtype)
    umax = np.max(np.hypot(rux, ruy))
    err = np.max(np.hypot(ux - rux, uy - ruy)) / umax
    l2 = float(np.sqrt(np.sum((ux - rux) ** 2 + (uy - ruy) ** 2) / np.sum(rux ** 2 + ruy ** 2)))
    print(f"PARITY {{\"case\": \"cavity 48x40 {dtype}\", \"vel_max\": {err:.3e}, \"vel_l2\": {l2:.3e}}}")
    assert l2 <= tol_l2 and err <= tol_max, (l2, err)


def test_cavity_128_2000_steps_fp32():
    """Lid-driven cavity 128x128, tau 0.6, lid 0.05, 2000 steps, FP32 against the FP64 oracle."""
    n = 128
    flags = lbm.gen_cavity(n, n)
    f0 = oracle.d2q9_equilibrium(np.ones((n, n)), np.zeros((n, n)), np.zeros((n, n)))
    ref = oracle.d2q9_run(f0, flags, 0.6, 2000, wall_velocity=(0.05, 0))
    _, rux, ruy = oracle.d2q9_moments(ref, flags, wall_velocity=(0.05, 0))
    with lbm.Lattice(n, n, tau=0.6, wall_velocity=(0.05, 0, 0)) as L:
        L.set_flags(flags)
        L.init_equilibrium()
        L.step(2000)
        _, ux, uy = L.moments()
    umax = np.max(np.hypot(rux, ruy))
    err = np.max(np.hypot(ux - rux, uy - ruy)) / umax
    assert err < 1e-4, err


def test_mass_conservation_fp32_channel():
    nx, ny = 256, 64
    flags, _ = lbm.gen_channel(nx, ny, 4, 3, 6, 9)
    with lbm.Lattice(nx, ny, tau=0.55, periodic=1) as L:
        L.set_flags(flags)
        L.init_equilibrium()
        m0 = L.conservation()
        L.step(500)
        m1 = L.conservation()
    assert abs(m1[0] - m0[0]) / m0[0] < 1e-6


def test_population_and_aos_round_trip():
    nx, ny = 35, 18
    f0 = random_state(nx, ny, 5)
    with lbm.Lattice(nx, ny, dtype="f32") as L:
        L.load_populations(f0.astype(np.float32))
        back = L.retrieve_populations()
        assert np.max(np.abs(back - f0)) < 1e-7
        aos = L.retrieve_aos()
        # record index y + ny*x, populations in the in-plane reference slots
        recs = aos.reshape(nx, ny)
        for q, slot in enumerate(lbm.capi.AOS_SLOTS_D2Q9):
            assert np.allclose(recs["f"][:, :, slot].T, back[q], atol=0)
        assert np.array_equal(recs["x"], np.repeat(np.arange(nx)[:, None], ny, 1))
        L2 = lbm.Lattice(nx, ny, dtype="f32")
        L2.load_aos(aos)
        assert np.max(np.abs(L2.retrieve_populations() - back)) < 1e-7
        L2.close()


def test_invalid_flags_rejected():
    with lbm.Lattice(8, 8) as L:
        bad = np.zeros((8, 8), np.uint8)
        bad[3, 3] = 7
        with pytest.raises(lbm.LBMError):
            L.set_flags(bad)
        with pytest.raises(lbm.LBMError):
            L.load_populations(np.zeros(5))
        with pytest.raises(lbm.LBMError):
            L.step(-1)


def test_steps_are_deterministic():
    nx, ny = 96, 40
    flags, _ = lbm.gen_channel(nx, ny, 3, 3, 5, 2)
    outs = []
    for _ in range(2):
        with lbm.Lattice(nx, ny, tau=0.55, periodic=1, body_force=(1e-5, 0, 0)) as L:
            L.set_flags(flags)
            L.init_equilibrium()
            L.step(100)
            outs.append(L.retrieve_populations())
    assert np.array_equal(outs[0], outs[1])


# (cells per thread, block width, rows per block, L2 policy)
# (cells per thread, block width, rows per block, L2 policy); cells per thread 0 is the bulk-copy
# pipeline of 16-bit storage (160 threads, 4 cells per consumer thread, one row per task; the last
# field the ring variant)
SHAPES = [(1, 256, 1, 0), (1, 128, 2, 0), (2, 64, 1, 0), (2, 32, 4, 1), (4, 32, 1, 2), (4, 64, 2, 0),
          (4, 128, 1, 1), (8, 32, 1, 1), (8, 64, 2, 2), (0, 160, 1, 0), (0, 160, 1, 1), (0, 160, 1, 2),
          (-2, 64, 8, 0), (-2, 64, 16, 0), (-2, 128, 8, 0),   # -2: two steps per launch on shared-memory tiles
          (-3, 64, 4, 0), (-3, 64, 8, 0)]                       # -3: the same with persistent blocks


def shape_ok(dtype, v):
    return v == 1 or (dtype == "f32" and v in (2, 4, -2, -3)) or \
        (dtype in ("f16s", "bf16s") and v in (0, 2, 4, 8, -2, -3)) or (dtype == "f64" and v == 2)


@pytest.mark.parametrize("shape", SHAPES)
@pytest.mark.parametrize("name", ["closed_box", "channel_force", "cavity_lid", "periodic_xy_force", "open_edges",
                                  "periodic_y_moving"])
def test_every_launch_shape_fp64_exact(name, shape):
    """Scalar and vectorised paths (odd widths, wrap and walls inside and at the edges of a vector,
    solid cells inside vectors) all match the FP64 oracle."""
    if not shape_ok("f64", shape[0]):
        pytest.skip("shape not available for FP64 storage")
    nx, ny, builder, periodic, force, wall, tau, steps = CASES[name]
    (tau,), force, wall = f32(tau), f32(*force), f32(*wall)
    flags = build_flags(name, nx, ny, builder)
    f0 = random_state(nx, ny, zlib.crc32(name.encode()))
    ref = oracle.d2q9_run(f0, flags, tau, steps, periodic=periodic, force=force, wall_velocity=wall)
    with lbm.Lattice(nx, ny, dtype="f64", tau=tau, periodic=periodic, body_force=(*force, 0),
                     wall_velocity=(*wall, 0)) as L:
        L.set_flags(flags)
        L.load_populations(f0)
        L.set_launch(*shape)
        L.step(steps)
        got = L.retrieve_populations(np.float64)
    fluid = flags == 0
    assert np.max(np.abs(got - ref)[:, fluid]) <= 1e-12
    # solid cells keep their initial populations in both buffers
    assert np.array_equal(got[:, ~fluid], f0[:, ~fluid]) or np.max(np.abs(got - f0)[:, ~fluid]) < 1e-15


@pytest.mark.parametrize("dtype", ["f32", "f16s", "bf16s"])
def test_shapes_and_sweep_orders_agree_bitwise(dtype):
    """The update of a cell does not depend on the launch shape or on the row order: every shape
    and both sweep orders give bit-identical populations."""
    nx, ny = 203, 77
    flags, _ = lbm.gen_channel(nx, ny, 5, 3.0, 7.0, 4)
    flags[ny // 2, :] = np.where(np.arange(nx) % 9 == 0, lbm.MOVING_WALL, flags[ny // 2, :])
    outs = {}
    for shape in SHAPES:
        if not shape_ok(dtype, shape[0]):
            continue
        for alt in (True, False):
            with lbm.Lattice(nx, ny, dtype=dtype, tau=0.58, periodic=1, body_force=(2e-5, 1e-6, 0),
                             wall_velocity=(0.02, 0, 0)) as L:
                L.set_flags(flags)
                L.init_equilibrium()
                L.set_launch(*shape)
                L.set_sweep_alternation(alt)
                L.step(41)
                outs[(shape, alt)] = L.retrieve_populations()
    first = next(iter(outs.values()))
    for k, v in outs.items():
        assert np.array_equal(v, first), k


@pytest.mark.parametrize("dtype", ["f16s", "bf16s"])
@pytest.mark.parametrize("periodic", [0, 1, 2, 3])
def test_bulk_pipeline_matches_vector_kernel_across_strips(dtype, periodic):
    """The bulk-copy pipeline over several strips and row runs (strip edges, run edges, wrap
    in x and y, walls, moving walls, solid cells on strip edges) is bit-identical to the vector
    kernel."""
    nx, ny = 777, 70
    flags, _ = lbm.gen_channel(nx, ny, 9, 3.0, 9.0, 11)
    if periodic & 2:
        flags[0, :] = flags[-1, :] = 0
    flags[:, 510:514] = np.where(np.arange(ny)[:, None] % 5 == 0, 1, flags[:, 510:514])  # solid on a strip edge
    flags[ny // 3, ::7] = lbm.MOVING_WALL
    f0 = random_state(nx, ny, 5 + periodic)
    outs = []
    for shape in ((8, 64, 2, 0), (0, 160, 1, 0), (0, 160, 1, 1), (0, 160, 1, 2)):
        with lbm.Lattice(nx, ny, dtype=dtype, tau=0.61, periodic=periodic, body_force=(1e-5, -2e-6, 0),
                         wall_velocity=(0.03, 0.01, 0)) as L:
            L.set_flags(flags)
            L.load_populations(f0)
            L.set_launch(*shape)
            L.step(23)
            outs.append(L.retrieve_populations())
    for o in outs[1:]:
        assert np.array_equal(o, outs[0])


def test_autotune_picks_a_valid_shape_and_keeps_state():
    nx, ny = 512, 256
    flags, _ = lbm.gen_channel(nx, ny, 6, 4, 9, 8)
    with lbm.Lattice(nx, ny, tau=0.6, periodic=1) as L:
        L.set_flags(flags)
        L.init_equilibrium()
        before = L.retrieve_populations()
        v, tx, ty, pol = L.autotune(retune=True)
        if v == -2:  # two steps per launch on tiles of tx x ty cells
            assert (tx, ty) in ((64, 8), (64, 16), (128, 8)) and pol == 0
        elif v == -3:  # the same with persistent blocks
            assert (tx, ty) in ((64, 4), (64, 8)) and pol == 0
        else:
            assert v in (1, 2, 4) and tx % 32 == 0 and tx * ty <= 256 and pol in (0, 1, 2)
        assert L.info()["tuned"] == 1
        assert np.array_equal(L.retrieve_populations(), before)  # tuning leaves the state alone


def test_bad_launch_shape_rejected():
    with lbm.Lattice(64, 8, dtype="f64") as L:
        with pytest.raises(lbm.LBMError):
            L.set_launch(1, 64, 1, 1)  # the scalar path has no L2 hints
        with pytest.raises(lbm.LBMError):
            L.set_launch(4, 64, 1)  # FP64 vectors are 2 wide
        with pytest.raises(lbm.LBMError):
            L.set_launch(2, 48, 1)  # not a multiple of 32
        with pytest.raises(lbm.LBMError):
            L.set_launch(2, 256, 2)  # more than 256 threads
        with pytest.raises(lbm.LBMError):
            L.set_launch(0, 160, 8)  # the bulk-copy pipeline is for 16-bit storage
    with lbm.Lattice(64, 8, dtype="f16s") as L:
        with pytest.raises(lbm.LBMError):
            L.set_launch(0, 64, 1)  # the bulk-copy pipeline has 160 threads per block
        with pytest.raises(lbm.LBMError):
            L.set_launch(0, 160, 1, 3)  # three pipeline variants
        with pytest.raises(lbm.LBMError):
            L.set_launch(0, 160, 2, 0)  # one row per task


@pytest.mark.parametrize("dtype", ["f16s", "f32"])
def test_domain_past_32bit_indexing_reproduces_its_tile(dtype):
    """A 16384 x 14592 domain (9 planes x 239 M cells: offsets past 2^31, so the step runs with
    64-bit indexing) periodic in both directions, with flags that repeat a 64 x 64 tile, started at
    equilibrium: every 64 x 64 tile of its density and velocity equals, bit for bit, the 64 x 64
    domain run alone (size-independent check of the large-index path), and its conserved sums are
    58,368 times the tile's."""
    tile = 64
    t_flags = np.zeros((tile, tile), np.uint8)
    yy, xx = np.mgrid[0:tile, 0:tile]
    t_flags[(xx - 30.5) ** 2 + (yy - 33.5) ** 2 < 10.0 ** 2] = 1
    t_flags[5, 50:54] = lbm.MOVING_WALL
    kw = dict(dtype=dtype, tau=0.6, periodic=3, body_force=(1e-5, 2e-6, 0), wall_velocity=(0.02, 0, 0))
    steps = 7
    with lbm.Lattice(tile, tile, **kw) as L:
        L.set_flags(t_flags)
        L.init_equilibrium()
        L.step(steps)
        want = L.moments()
        want_cons = L.conservation()
    nx, ny = 16384, 14592
    assert 9 * nx * ny > 2 ** 31
    with lbm.Lattice(nx, ny, **kw) as L:
        L.set_flags(np.tile(t_flags, (ny // tile, nx // tile)))
        L.init_equilibrium()
        L.step(steps)
        cons = L.conservation()
        got = L.moments()
    ntiles = (nx // tile) * (ny // tile)
    for g, w in zip(got, want):
        g4 = g.reshape(ny // tile, tile, nx // tile, tile)
        assert np.array_equal(g4, np.broadcast_to(w[None, :, None, :], g4.shape))
    for c, w in zip(cons[:3], want_cons[:3]):
        assert abs(c - ntiles * w) <= 1e-9 * max(1.0, abs(ntiles * w))


@pytest.mark.parametrize("periodic", [0, 1])
def test_bulk_pipeline_wait_gives_up_and_the_context_recovers(periodic):
    """The bulk-copy pipeline's bounded waits, exercised without any fault: with a 1 ms limit and the
    copies of one task left out, the consumer warps' wait for that slot runs out, the block records
    the timeout and exits, and the next synchronisation returns LBM_ERR_TIMEOUT.  The context stays
    usable: with the defaults back and the populations reloaded, its steps equal, bit for bit, the
    vector kernel's on a fresh context."""
    nx, ny = 777, 70
    flags, _ = lbm.gen_channel(nx, ny, 9, 3.0, 9.0, 11)
    f0 = random_state(nx, ny, 17)
    kw = dict(dtype="f16s", tau=0.61, periodic=periodic, body_force=(1e-5, 0, 0))
    with lbm.Lattice(nx, ny, **kw) as L:
        L.set_flags(flags)
        L.load_populations(f0)
        L.set_launch(0, 160, 1, 0)
        L.set_pipeline_wait(1_000_000, skip_task=5)
        L.step(3)
        with pytest.raises(lbm.LBMError) as err:
            L.synchronize()
        assert err.value.status == lbm.capi.ERR_TIMEOUT and "bounded wait" in str(err.value)
        L.synchronize()  # the status was taken: nothing left to report
        L.set_pipeline_wait()
        L.load_populations(f0)
        L.step(23)
        got = L.retrieve_populations()
    with lbm.Lattice(nx, ny, **kw) as R:
        R.set_flags(flags)
        R.load_populations(f0)
        R.set_launch(8, 64, 2, 0)
        R.step(23)
        want = R.retrieve_populations()
    assert np.array_equal(got, want)


def test_pipeline_wait_arguments_checked():
    with lbm.Lattice(64, 8, dtype="f16s") as L:
        with pytest.raises(lbm.LBMError):
            L.set_pipeline_wait(10)  # below 1 microsecond
        with pytest.raises(lbm.LBMError):
            L.set_pipeline_wait(1_000_000, skip_task=-2)


@pytest.mark.parametrize("shape", [(1, 256, 1, 0), (2, 64, 1, 0), (2, 32, 4, 0)])
def test_solid_cells_stay_frozen_across_flag_changes(shape):
    """The step kernels never write a solid cell; both population buffers hold its values (the link
    build copies solid cells into the other buffer, so flags can change between steps).  FP64 against
    the oracle, which copies solid cells forward, on every cell -- solid ones included -- after 5
    steps with one set of flags and 7 (an odd count: the other buffer is current) with another that
    adds a disk and frees part of an old one."""
    nx, ny = 97, 41
    a = np.zeros((ny, nx), np.uint8)
    a[0, :] = a[-1, :] = 1
    yy, xx = np.mgrid[0:ny, 0:nx]
    a[(xx - 30) ** 2 + (yy - 20) ** 2 <= 36] = 1
    b = a.copy()
    b[(xx - 70) ** 2 + (yy - 18) ** 2 <= 25] = 1       # a new disk
    b[(xx - 30) ** 2 + (yy - 20) ** 2 <= 36] = 0
    b[(xx - 30) ** 2 + (yy - 20) ** 2 <= 9] = 1        # the old disk shrinks
    f0 = random_state(nx, ny, 4242)
    # the library takes tau and the force as float: the oracle gets the same values
    tau, force = float(np.float32(0.7)), (float(np.float32(2e-6)), 0.0)
    ref = oracle.d2q9_run(f0, a, tau, 5, periodic=1, force=force)
    ref = oracle.d2q9_run(ref, b, tau, 7, periodic=1, force=force)
    with lbm.Lattice(nx, ny, dtype="f64", tau=tau, periodic=1, body_force=(*force, 0)) as L:
        L.set_flags(a)
        L.load_populations(f0)
        L.set_launch(*shape)
        L.step(5)
        L.set_flags(b)
        L.step(7)
        got = L.retrieve_populations(np.float64)
    assert np.max(np.abs(got - ref)) <= 1e-12
    solid = b != 0
    frozen = (a != 0) & solid
    assert np.array_equal(got[:, frozen], f0[:, frozen])  # solid throughout: the initial values


@pytest.mark.parametrize("dtype", ["f32", "f16s"])
@pytest.mark.parametrize("periodic", [0, 1, 2, 3])
def test_two_step_tiles_match_the_one_step_kernel(dtype, periodic):
    """Two steps per launch on shared-memory tiles (walls, moving walls, solid cells on tile edges,
    wrap in x and y, domains smaller than a tile, an odd step count) give the one-step vector
    kernel's populations bit for bit."""
    for nx, ny in ((777, 70), (5, 3), (64, 8), (130, 17)):
        flags, _ = lbm.gen_channel(nx, ny, 4 if nx > 60 else 0, 2.0, 6.0, 13) if nx > 8 else \
            (np.zeros((ny, nx), np.uint8), None)
        if periodic & 2:
            flags[0, :] = flags[-1, :] = 0
        if nx > 64:
            flags[:, 63:65] = np.where(np.arange(ny)[:, None] % 4 == 0, 1, flags[:, 63:65])  # solid on a tile edge
            flags[ny // 3, ::5] = lbm.MOVING_WALL
        f0 = random_state(nx, ny, 31 + periodic + nx)
        outs = []
        for shape in ((2, 64, 1, 0), (-2, 64, 8, 0), (-2, 64, 16, 0), (-2, 128, 8, 0), (-3, 64, 4, 0), (-3, 64, 8, 0)):
            with lbm.Lattice(nx, ny, dtype=dtype, tau=0.57, periodic=periodic, body_force=(1e-5, -3e-6, 0),
                             wall_velocity=(0.03, 0.01, 0)) as L:
                L.set_flags(flags)
                L.load_populations(f0)
                L.set_launch(*shape)
                L.step(6)
                L.step(17)
                outs.append(L.retrieve_populations())
        for k, o in enumerate(outs[1:]):
            assert np.array_equal(o, outs[0]), (nx, ny, k)
