"""D3Q27_REF parity through the C ABI.

1. The reference's own known-answer tests (test/CalculationsTest.cpp, test/CoordinatesTest.cpp),
   rebuilt on the library: same set-up, same expected values (tests/golden/).
2. Seeded random lattices against the CPU restatement of the reference kernels (oracle/), for every
   single pass and for whole steps in both step orders.  Tolerance: max |f_gpu - f_oracle| <=
   1e-5 * max |f_oracle| (float rounding of the FP32 sums and of the unordered reflection adds).
"""
import numpy as np
import pytest

import latticeboltzmanncuda_gb300 as lbm
import oracle
from conftest import known
from refcases import INTERNAL, REFLECTED, SOURCE, cell, pack_dir, reflections_case
from test_oracle_golden import check_force

pytestmark = pytest.mark.gpu

REF = dict(mode="d3q27_ref", dtype="f32")


def lattice(dims, tau=1.0, order=lbm.ORDER_STREAM_COLLIDE, force_mode=lbm.FORCE_REFERENCE):
    return lbm.Lattice(*dims, tau=tau, order=order, force_mode=force_mode, **REF)


def near(a, rec):
    assert abs(float(a) - rec["value"]) <= rec["tol"], (a, rec)


# ------------------------------------------------------------------ known answers (AoS path)
def test_streaming(golden):
    # CalculationsTest.cpp:19-45
    with lattice((1, 2, 1)) as L:
        pts = np.zeros(2, lbm.LATTICE_POINT)
        pts[0]["f"][5] = 2.0
        L.load_aos(pts)
        L.apply(lbm.OP_STREAM)
        out = L.retrieve_aos()
    near(out[1]["f"][5], known(golden, "CalculationsTest.TestStreaming", 44))


def test_collision(golden):
    # CalculationsTest.cpp:47-75
    with lattice((1, 1, 1)) as L:
        pts = np.zeros(1, lbm.LATTICE_POINT)
        pts[0]["f"][0] = 2.0
        L.load_aos(pts)
        L.apply(lbm.OP_COLLIDE)
        out = L.retrieve_aos()
    for q, line in ((0, 72), (1, 73), (2, 74)):
        near(out[0]["f"][q], known(golden, "CalculationsTest.TestCollision", line))


def test_full(golden):
    # CalculationsTest.cpp:77-105 (Lattice::simulateLattice = stream, collide)
    with lattice((1, 2, 1)) as L:
        pts = np.zeros(2, lbm.LATTICE_POINT)
        pts[0]["f"][5] = 2.0
        L.load_aos(pts)
        L.step(1)
        out = L.retrieve_aos()
    for q, line in ((0, 102), (1, 103), (2, 104)):
        near(out[1]["f"][q], known(golden, "CalculationsTest.TestFull", line))


@pytest.mark.parametrize("with_force", [False, True])
def test_reflections(golden, with_force):
    # CalculationsTest.cpp:107-146 and 148-197
    dims, f, flags, tab_idx, tabs = reflections_case(golden)
    name = "CalculationsTest.TestReflectionsData" if with_force else "CalculationsTest.TestReflections"
    lines = (186, 187, 188, 190) if with_force else (141, 142, 143, 145)
    with lattice(dims) as L:
        pts = np.zeros(27, lbm.LATTICE_POINT)
        pts["f"] = f
        pts["isInternal"] = (flags & INTERNAL) != 0
        pts["isReflected"] = (flags & REFLECTED) != 0
        L.load_aos(pts)
        L.set_reflection_tables(np.nonzero(tab_idx >= 0)[0], tabs)
        if with_force:
            L.set_force((0, 0, 0), True)
        L.apply(lbm.OP_REFLECT)
        out = L.retrieve_aos()
        force = L.get_force()
    near(out[cell(dims, 2, 1, 2)]["f"][17], known(golden, name, lines[0]))
    near(out[cell(dims, 1, 1, 2)]["f"][4], known(golden, name, lines[1]))
    near(out[cell(dims, 2, 2, 2)]["f"][26], known(golden, name, lines[2]))
    near(out[cell(dims, 1, 1, 1)]["f"][1], known(golden, name, lines[3]))
    assert out[cell(dims, 1, 1, 1)]["isInternal"] and out[cell(dims, 1, 1, 1)]["isReflected"]
    if with_force:
        check_force(golden, force)


@pytest.mark.parametrize("plane", [False, True])
def test_flow_generation(golden, plane):
    # CalculationsTest.cpp:199-234 (point criterion) and 236-277 (plane x = 0)
    dims = (3, 3, 3)
    mask = np.zeros(27, np.uint8)
    if plane:
        for y in range(3):
            for z in range(3):
                mask[cell(dims, 0, y, z)] = 1
    else:
        mask[cell(dims, 1, 1, 1)] = 1
    induced = np.zeros(27, np.float32)
    induced[0] = 1.0
    with lattice(dims) as L:
        L.load_aos(np.zeros(27, lbm.LATTICE_POINT))
        L.set_flow(mask, induced)
        L.apply(lbm.OP_FLOW)
        out = L.retrieve_aos()
    if plane:
        for y in range(3):
            for z in range(3):
                near(out[cell(dims, 0, y, z)]["f"][0], known(golden, "CalculationsTest.TestPlaneFlowGeneration", 273))
                near(out[cell(dims, 1, y, z)]["f"][0], known(golden, "CalculationsTest.TestPlaneFlowGeneration", 274))
    else:
        near(out[cell(dims, 1, 1, 1)]["f"][0], known(golden, "CalculationsTest.TestFlowGeneration", 232))
        near(out[cell(dims, 0, 0, 0)]["f"][0], known(golden, "CalculationsTest.TestFlowGeneration", 233))


def test_load_and_retrieve_coordinates():
    # CoordinatesTest.cpp:14-32 and 34-86: records round-trip, coordinates follow z + Z*(y + Y*x)
    n = 40
    with lattice((n, n, n)) as L:
        pts = np.zeros(n ** 3, lbm.LATTICE_POINT)
        x, y, z = np.meshgrid(np.arange(n), np.arange(n), np.arange(n), indexing="ij")
        pts["x"], pts["y"], pts["z"] = x.ravel(), y.ravel(), z.ravel()
        pts["f"][:, 5] = np.arange(n ** 3, dtype=np.float32)
        L.load_aos(pts)
        out = L.retrieve_aos()
    assert np.array_equal(out["x"], pts["x"]) and np.array_equal(out["y"], pts["y"]) and np.array_equal(out["z"], pts["z"])
    assert np.array_equal(out["f"], pts["f"])


# ------------------------------------------------------------------ seeded parity vs the oracle
def random_lattice(dims, seed, solid=0.2):
    """Random populations, internal cells, reflection tables (targets always non-internal, as
    Lattice::preProcessModel builds them, Lattice.cpp:356-369) and a flow-source plane."""
    X, Y, Z = dims
    n = X * Y * Z
    rng = np.random.default_rng(seed)
    f = rng.random((n, 27), dtype=np.float32) * 0.05
    internal = rng.random(n) < solid
    flags = np.where(internal, INTERNAL, 0).astype(np.uint8)
    C = oracle.C27
    cells, recs = [], []
    for c in np.nonzero(internal)[0]:
        x, y, z = c // (Y * Z), (c // Z) % Y, c % Z
        ok = []
        for d in range(1, 27):
            tx, ty, tz = x + C[d, 0], y + C[d, 1], z + C[d, 2]
            if 0 <= tx < X and 0 <= ty < Y and 0 <= tz < Z and not internal[tz + Z * (ty + Y * tx)]:
                ok.append(d)
        if not ok:
            continue
        flags[c] |= REFLECTED
        rec = np.zeros(1, lbm.REFLECTION_VALUES)[0]
        for p in range(27):
            k = rng.integers(1, 4)
            dirs = rng.choice(ok, size=min(k, len(ok)), replace=False)
            w = rng.random(len(dirs)).astype(np.float32)
            w /= w.sum()
            for j, d in enumerate(dirs):
                s = 3 * p + j
                pack_dir(rec, s, int(d))
                rec["w"][s] = w[j]
        cells.append(c)
        recs.append(rec)
    src = np.zeros(n, np.uint8)
    src[: Y * Z] = 1  # plane x = 0
    flags |= np.where(src > 0, SOURCE, 0).astype(np.uint8)
    induced = (rng.random(27) * 1e-3).astype(np.float32)
    return f, flags, np.array(cells, np.int32), np.array(recs, lbm.REFLECTION_VALUES), induced


def tab_index(n, cells):
    t = np.full(n, -1, np.int32)
    t[cells] = np.arange(len(cells), dtype=np.int32)
    return t


def close(got, ref):
    scale = max(float(np.max(np.abs(ref))), 1e-30)
    err = float(np.max(np.abs(got - ref)))
    assert err <= 1e-5 * scale, (err, scale)


DIMS = [(6, 5, 6), (9, 7, 9), (4, 12, 4)]


@pytest.mark.parametrize("dims", DIMS)
@pytest.mark.parametrize("force_mode", [lbm.FORCE_REFERENCE, lbm.FORCE_MOMENTUM_EXCHANGE])
def test_single_passes_match_oracle(dims, force_mode):
    f, flags, cells, recs, induced = random_lattice(dims, sum(dims) * 7 + force_mode)
    n = f.shape[0]
    ti = tab_index(n, cells)
    with lattice(dims, tau=0.8, force_mode=force_mode) as L:
        L.set_flags(flags)
        L.set_reflection_tables(cells, recs)
        L.set_flow(flags & SOURCE, induced)
        L.set_force((0.1, -0.2, 0.3), True)
        L.load_populations(f)
        # stream
        L.apply(lbm.OP_STREAM)
        ref = oracle.d3q27_stream(dims, f)
        close(L.retrieve_populations(), ref)
        # reflect (+ force)
        L.apply(lbm.OP_REFLECT)
        force = np.array([0.1, -0.2, 0.3], np.float32)
        ref = oracle.d3q27_reflect(dims, ref, flags, ti, recs, force=force, force_mode=force_mode)
        close(L.retrieve_populations(), ref)
        assert np.allclose(L.get_force(), force, rtol=1e-5, atol=1e-6)
        # collide
        L.apply(lbm.OP_COLLIDE)
        ref = oracle.d3q27_collide(dims, ref, 0.8)
        close(L.retrieve_populations(), ref)
        # flow
        L.apply(lbm.OP_FLOW)
        ref = oracle.d3q27_flow(dims, ref, flags, induced)
        close(L.retrieve_populations(), ref)


@pytest.mark.parametrize("dims", DIMS)
@pytest.mark.parametrize("order", [lbm.ORDER_STREAM_COLLIDE, lbm.ORDER_CLI])
def test_fused_steps_match_oracle(dims, order):
    f, flags, cells, recs, induced = random_lattice(dims, sum(dims) + order)
    n = f.shape[0]
    ti = tab_index(n, cells)
    steps = 6
    with lattice(dims, tau=0.7, order=order) as L:
        L.set_flags(flags)
        L.set_reflection_tables(cells, recs)
        L.set_flow(flags & SOURCE, induced)
        L.set_force((0, 0, 0), True)
        L.load_populations(f)
        L.step(steps)
        got = L.retrieve_populations()
        force = L.get_force()
    ref_force = np.zeros(3, np.float32)
    ref = oracle.d3q27_run(dims, f, flags, 0.7, steps, order=order, tab_idx=ti, tabs=recs,
                           induced=induced, force=ref_force, force_mode=0)
    close(got, ref)
    if order == lbm.ORDER_CLI:
        assert np.allclose(force, ref_force, rtol=1e-5, atol=1e-6)


def test_moments_and_conservation():
    dims = (5, 4, 6)
    f, flags, _, _, _ = random_lattice(dims, 3, solid=0.0)
    with lattice(dims) as L:
        L.load_populations(f)
        rho, ux, uy, uz = L.moments()
        cons = L.conservation()
    C = oracle.C27.astype(np.float64)
    split = np.array([0] + [1] * 6 + [0.5] * 12 + [1 / 3] * 8)
    assert np.allclose(rho, f.sum(1), rtol=1e-6)
    assert np.allclose(ux, (f * C[:, 0] * split).sum(1) / f.sum(1), rtol=1e-5, atol=1e-7)
    assert np.allclose(cons[0], f.astype(np.float64).sum(), rtol=1e-12)
    assert np.allclose(cons[1:], (f.astype(np.float64) @ C).sum(0), rtol=1e-9, atol=1e-9)


def test_rejects_bad_tables():
    dims = (3, 3, 3)
    with lattice(dims) as L:
        rec = np.zeros(1, lbm.REFLECTION_VALUES)
        pack_dir(rec[0], 4, 30)
        flags = np.zeros(27, np.uint8)
        flags[13] = INTERNAL | REFLECTED
        L.set_flags(flags)
        with pytest.raises(lbm.LBMError):
            L.set_reflection_tables([13], rec)
        with pytest.raises(lbm.LBMError):
            L.set_reflection_tables([13, 13], np.zeros(2, lbm.REFLECTION_VALUES))
        with pytest.raises(lbm.LBMError):
            L.set_reflection_tables([99], np.zeros(1, lbm.REFLECTION_VALUES))


# ------------------------------------------------------------------ mesh front end + library
@pytest.mark.parametrize("with_force", [False, True])
def test_reflections_from_mesh(golden, with_force):
    """CalculationsTest.cpp:107-197 with the flags and tables built by the mesh front end
    (insertModel + preProcessModel) and the reflection pass on the GPU; the force meets the
    reference's own 1e-6 bound."""
    from test_mesh_front_end import golden_mesh
    dims = (3, 3, 3)
    m = golden_mesh(golden, "cube_angled.obj")
    flags, _ = m.rasterize(dims, 0.5)
    cells, recs, flags = m.reflection_tables(dims, 0.5, flags)
    f = np.zeros((27, 27), np.float32)
    f[cell(dims, 1, 1, 1), 1] = 1.0
    name = "CalculationsTest.TestReflectionsData" if with_force else "CalculationsTest.TestReflections"
    lines = (186, 187, 188, 190) if with_force else (141, 142, 143, 145)
    with lattice(dims) as L:
        L.set_flags(flags)
        L.load_populations(f)
        L.set_reflection_tables(cells, recs)
        if with_force:
            L.set_force((0, 0, 0), True)
        L.apply(lbm.OP_REFLECT)
        out = L.retrieve_populations()
        force = L.get_force()
    for (x, y, z, q), line in zip(((2, 1, 2, 17), (1, 1, 2, 4), (2, 2, 2, 26), (1, 1, 1, 1)), lines):
        near(out[cell(dims, x, y, z), q], known(golden, name, line))
    if with_force:
        for k, line in enumerate((194, 195, 196)):
            near(force[k], known(golden, "CalculationsTest.TestReflectionsData", line))


def test_sphere_mesh_steps_match_oracle():
    """A sphere mesh rasterised on 20^3, its tables from the front end, 5 CLI-order steps with the
    force: library vs CPU oracle."""
    from refcases import icosphere
    dims = (20, 20, 20)
    verts, faces = icosphere(2, 0.3, (0.5, 0.5, 0.5))
    m = lbm.Mesh.from_arrays(verts, faces)
    flags, applied = m.rasterize(dims, 1 / 19)
    assert applied
    cells, recs, flags = m.reflection_tables(dims, 1 / 19, flags)
    assert len(cells) > 100
    n = 20 ** 3
    rng = np.random.default_rng(8)
    f = (rng.random((n, 27), dtype=np.float32) * 0.05).astype(np.float32)
    flags[: 20 * 20] |= SOURCE
    induced = (rng.random(27) * 1e-3).astype(np.float32)
    tab_idx = np.full(n, -1, np.int32)
    tab_idx[cells] = np.arange(len(cells), dtype=np.int32)
    force_ref = np.zeros(3, np.float32)
    ref = oracle.d3q27_run(dims, f, flags, 0.8, 5, order=lbm.ORDER_CLI, tab_idx=tab_idx, tabs=recs,
                           induced=induced, force=force_ref, force_mode=lbm.FORCE_REFERENCE)
    with lattice(dims, tau=0.8, order=lbm.ORDER_CLI) as L:
        L.set_flags(flags)
        L.load_populations(f)
        L.set_reflection_tables(cells, recs)
        L.set_flow(flags & SOURCE, induced)
        L.set_force((0, 0, 0), True)
        L.step(5)
        got = L.retrieve_populations()
        force = L.get_force()
    close(got, ref)
    assert np.max(np.abs(force - force_ref)) <= 1e-5 * max(1e-30, float(np.max(np.abs(force_ref))))


def test_force_series_equals_per_step_reads():
    """lbm_step_force_series records the same running force as one lbm_step + lbm_get_force per
    step (the reference CLI's print loop), and leaves the same populations."""
    dims = (9, 7, 9)
    f, flags, cells, recs, induced = random_lattice(dims, 31)
    start = np.array([0.25, 0.0, -0.5], np.float32)

    def make():
        L = lattice(dims, tau=0.8, order=lbm.ORDER_CLI)
        L.set_flags(flags)
        L.load_populations(f)
        L.set_reflection_tables(cells, recs)
        L.set_flow(flags & SOURCE, induced)
        L.set_force(start, True)
        return L

    with make() as A, make() as B:
        series = A.step_force_series(7)
        per_step = []
        for _ in range(7):
            B.step(1)
            per_step.append(B.get_force())
        assert np.array_equal(series, np.array(per_step, np.float32))
        assert np.array_equal(A.retrieve_populations(), B.retrieve_populations())
        assert not np.array_equal(series[0], start)


def test_set_order_switches_the_fused_step():
    dims = (6, 5, 6)
    f, flags, cells, recs, induced = random_lattice(dims, 41)
    with lattice(dims, tau=0.9) as L:
        L.set_flags(flags)
        L.load_populations(f)
        L.set_reflection_tables(cells, recs)
        L.set_flow(flags & SOURCE, induced)
        L.step(2)
        L.set_order(lbm.ORDER_CLI)
        L.step(3)
        got = L.retrieve_populations()
        with pytest.raises(lbm.LBMError):
            L.set_order(7)
    tab_idx = np.full(f.shape[0], -1, np.int32)
    tab_idx[cells] = np.arange(len(cells), dtype=np.int32)
    ref = oracle.d3q27_run(dims, f, flags, 0.9, 2, order=lbm.ORDER_STREAM_COLLIDE, tab_idx=tab_idx, tabs=recs,
                           induced=induced)
    ref = oracle.d3q27_run(dims, ref, flags, 0.9, 3, order=lbm.ORDER_CLI, tab_idx=tab_idx, tabs=recs, induced=induced)
    close(got, ref)


# ------------------------------------------------------------------ equilibrium evaluation
def test_equilibrium_selftest():
    """The float-float equilibrium (the single and the pair evaluator), wherever its error bound
    accepts it, equals the reference's FP64 evaluation bit for bit, over about 100 million
    evaluations with rho over 16 decades and |u| up to 2; for low-Mach draws (|u| <= 0.05) the
    FP64 fallback settles under 0.1 % of them."""
    import ctypes
    out = (ctypes.c_int64 * 2)()
    lbm.capi.check(lbm.capi.lib().lbm_d3q27_equilibrium_selftest(2_000_000, 20261203, 0, out))
    assert out[0] == 0, out[0]
    assert out[1] < 2_000_000 * 0.5 * 26 * 1e-3, out[1]


@pytest.mark.parametrize("order", [lbm.ORDER_STREAM_COLLIDE, lbm.ORDER_CLI])
def test_float_float_steps_equal_fp64_steps(order):
    dims = (12, 9, 12)
    f, flags, cells, recs, induced = random_lattice(dims, 77)
    f = f * 20.0  # larger populations and velocities than the default lattice
    outs, forces = [], []
    for fp64 in (False, True):
        with lattice(dims, tau=0.7, order=order) as L:
            L.set_equilibrium_evaluation(fp64)
            L.set_flags(flags)
            L.load_populations(f)
            L.set_reflection_tables(cells, recs)
            L.set_flow(flags & SOURCE, induced)
            L.set_force((0, 0, 0), True)
            L.step(9)
            outs.append(L.retrieve_populations())
            forces.append(L.get_force())
    assert np.array_equal(outs[0], outs[1])
    assert np.array_equal(forces[0], forces[1])


@pytest.mark.parametrize("tau", [0.5, 0.51, 0.55, 0.6, 0.7, 0.8, 0.9, 1.0, 1.2, 1.7, 3.0, 0.6180339887, 1e-3, 250.0])
def test_division_by_tau_matches_ieee_for_every_input(tau):
    """One Markstein correction of RN(x RN(1/tau)) gives the IEEE quotient for all 2^32 float x."""
    import ctypes
    bad = ctypes.c_int64(-1)
    lbm.capi.check(lbm.capi.lib().lbm_d3q27_division_check(ctypes.c_float(tau), 0, ctypes.byref(bad)))
    assert bad.value == 0
