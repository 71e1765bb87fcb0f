"""The library's D3Q27_REF mode against the reference's own CUDA kernels, run on the same GPU from a
cubin compiled from the reference sources (oracle/refkern.py, oracle/ref_harness.cpp).

Parity bar (as stated for this mode): flags bit-exact (the same bytes go to both), populations
within max |f_lib - f_ref| <= 1e-5 * max |f_ref| after the run, force within 1e-5 relative -- for the
default float-float equilibrium (the reference's FP64 value bit for bit) and for the FP32
equilibrium (LBM_EQ_FP32, a few ulps from it).
The reference's reflection scatter uses float atomics in no fixed order, so bit equality of the
populations is not expected.
"""
import numpy as np
import pytest

import latticeboltzmanncuda_gb300 as lbm
import oracle
from conftest import known
from refcases import INTERNAL, REFLECTED, SOURCE, cell, pack_dir, reflections_case
from test_gpu_d3q27_ref import close, random_lattice
from test_oracle_golden import check_force

pytestmark = pytest.mark.gpu

refkern = pytest.importorskip("oracle.refkern")
if not refkern.available():
    pytest.skip("reference kernels were not built (oracle/_ref/ref_kernels.cubin missing)", allow_module_level=True)


def points_from(f, flags):
    pts = np.zeros(f.shape[0], lbm.LATTICE_POINT)
    pts["f"] = f
    pts["isInternal"] = (flags & INTERNAL) != 0
    pts["isReflected"] = (flags & REFLECTED) != 0
    return pts


def near(a, rec):
    assert abs(float(a) - rec["value"]) <= rec["tol"], (a, rec)


# ------------------------------------------------------------------ the harness reproduces the reference tests
def test_reference_kernels_known_answers(golden):
    pts = np.zeros(2, lbm.LATTICE_POINT)
    pts[0]["f"][5] = 2.0
    out = refkern.run((1, 2, 1), pts, "S")
    near(out[1]["f"][5], known(golden, "CalculationsTest.TestStreaming", 44))
    out = refkern.run((1, 2, 1), pts, "SC")
    for q, line in ((0, 102), (1, 103), (2, 104)):
        near(out[1]["f"][q], known(golden, "CalculationsTest.TestFull", line))
    dims, f, flags, tab_idx, tabs = reflections_case(golden)
    force = np.zeros(3, np.float32)
    out = refkern.run(dims, points_from(f, flags), "R", tab_cells=np.nonzero(tab_idx >= 0)[0], tab_records=tabs,
                      force=force, threads=(3, 3, 3))
    near(out[cell(dims, 2, 1, 2)]["f"][17], known(golden, "CalculationsTest.TestReflectionsData", 186))
    near(out[cell(dims, 1, 1, 1)]["f"][1], known(golden, "CalculationsTest.TestReflectionsData", 190))
    check_force(golden, force)
    induced = np.zeros(27, np.float32)
    induced[0] = 1.0
    out = refkern.run((3, 3, 3), np.zeros(27, lbm.LATTICE_POINT), "F", flow_criterion=2, induced=induced)
    near(out[cell((3, 3, 3), 0, 2, 1)]["f"][0], known(golden, "CalculationsTest.TestPlaneFlowGeneration", 273))
    near(out[cell((3, 3, 3), 1, 2, 1)]["f"][0], known(golden, "CalculationsTest.TestPlaneFlowGeneration", 274))


# ------------------------------------------------------------------ library vs reference kernels
def restrict_slots(recs, max_pop):
    """Drop table slots of populations >= max_pop (the force comparison needs slots < 27)."""
    recs = recs.copy()
    for r in recs:
        for s in range(3 * max_pop, 81):
            pack_dir(r, s, 0)
            r["w"][s] = 0.0
    return recs


CASES = [((6, 5, 6), (1, 1, 6)), ((12, 8, 12), (2, 4, 12)), ((32, 16, 32), (1, 16, 32))]
EQ = ["float_float", "fp32"]  # equilibrium evaluations (lbm_set_equilibrium_evaluation)


@pytest.mark.parametrize("dims,threads", CASES)
@pytest.mark.parametrize("eq", EQ)
def test_stream_collide_matches_reference(dims, threads, eq):
    f, flags, cells, recs, _ = random_lattice(dims, 11 + dims[0])
    steps = 8
    # reflected cells carry their tables, as in a lattice prepared by Lattice::preProcessModel; the
    # stream-collide order does not read them
    ref = refkern.run(dims, points_from(f, flags), "SC", nsteps=steps, tau=0.75, tab_cells=cells,
                      tab_records=recs, threads=threads)
    with lbm.Lattice(*dims, mode="d3q27_ref", tau=0.75, order=lbm.ORDER_STREAM_COLLIDE) as L:
        L.set_equilibrium_evaluation(eq)
        L.load_aos(points_from(f, flags))
        L.step(steps)
        got = L.retrieve_aos()
    close(got["f"], ref["f"])
    assert np.array_equal(got["isInternal"], ref["isInternal"])
    assert np.array_equal(got["isReflected"], ref["isReflected"])


@pytest.mark.parametrize("dims,threads", CASES)
@pytest.mark.parametrize("eq", EQ)
def test_cli_order_matches_reference(dims, threads, eq):
    """stream, reflect, collide, flow (LatticeBoltzmannCuda.cpp:85-93) with mesh-style reflection
    tables on every slot and the flow plane x = 0 (FlowCriterion.cu:10-13)."""
    f, flags, cells, recs, induced = random_lattice(dims, 5 + dims[1])
    steps = 6
    ref = refkern.run(dims, points_from(f, flags), "SRCF", nsteps=steps, tau=0.7, tab_cells=cells,
                      tab_records=recs, flow_criterion=2, induced=induced, threads=threads)
    with lbm.Lattice(*dims, mode="d3q27_ref", tau=0.7, order=lbm.ORDER_CLI) as L:
        L.set_equilibrium_evaluation(eq)
        L.load_aos(points_from(f, flags))
        L.set_reflection_tables(cells, recs)
        L.set_flow(flags & SOURCE, induced)
        L.step(steps)
        got = L.retrieve_aos()
    close(got["f"], ref["f"])


@pytest.mark.parametrize("dims,threads", CASES[:2])
@pytest.mark.parametrize("eq", EQ)
def test_force_matches_reference(dims, threads, eq):
    f, flags, cells, recs, induced = random_lattice(dims, 17 + dims[2])
    recs = restrict_slots(recs, 9)
    start = np.array([0.5, -0.25, 0.125], np.float32)
    steps = 4
    ref_force = start.copy()
    ref = refkern.run(dims, points_from(f, flags), "SRCF", nsteps=steps, tau=0.9, tab_cells=cells,
                      tab_records=recs, flow_criterion=2, induced=induced, force=ref_force, threads=threads)
    with lbm.Lattice(*dims, mode="d3q27_ref", tau=0.9, order=lbm.ORDER_CLI) as L:
        L.set_equilibrium_evaluation(eq)
        L.load_aos(points_from(f, flags))
        L.set_reflection_tables(cells, recs)
        L.set_flow(flags & SOURCE, induced)
        L.set_force(start, True)
        L.step(steps)
        got = L.retrieve_aos()
        force = L.get_force()
    close(got["f"], ref["f"])
    assert np.max(np.abs(force - ref_force)) <= 1e-5 * np.max(np.abs(ref_force)), (force, ref_force)


@pytest.mark.parametrize("eq", EQ)
def test_separate_passes_match_reference(eq):
    """Lattice::simulateStreaming / simulateReflections / simulateCollision / simulateFlow one by one."""
    dims, threads = (9, 6, 9), (1, 2, 9)
    f, flags, cells, recs, induced = random_lattice(dims, 99)
    with lbm.Lattice(*dims, mode="d3q27_ref", tau=0.85) as L:
        L.set_equilibrium_evaluation(eq)
        L.load_aos(points_from(f, flags))
        L.set_reflection_tables(cells, recs)
        L.set_flow(flags & SOURCE, induced)
        pts = points_from(f, flags)
        for op, letter in ((lbm.OP_STREAM, "S"), (lbm.OP_REFLECT, "R"), (lbm.OP_COLLIDE, "C"), (lbm.OP_FLOW, "F")):
            pts = refkern.run(dims, pts, letter, tau=0.85, tab_cells=cells, tab_records=recs, flow_criterion=2,
                              induced=induced, threads=threads)
            L.apply(op)
            close(L.retrieve_aos()["f"], pts["f"])


@pytest.mark.parametrize("eq", EQ)
def test_sphere_mesh_cli_matches_reference(eq):
    """A sphere mesh through the front end (flags, tables), then 6 CLI-order steps: library vs the
    reference's own kernels on the same flags and tables (X == Z, grid tiled exactly)."""
    from refcases import icosphere
    dims, threads = (24, 16, 24), (1, 16, 24)
    verts, faces = icosphere(2, 0.25, (0.5, 0.34, 0.5))  # inside [0, 24/23] x [0, 16/23] x [0, 24/23]
    m = lbm.Mesh.from_arrays(verts, faces)
    spacing = 1 / 23
    flags, applied = m.rasterize(dims, spacing)
    assert applied
    cells, recs, flags = m.reflection_tables(dims, spacing, flags)
    assert len(cells) > 50
    n = int(np.prod(dims))
    rng = np.random.default_rng(21)
    f = (rng.random((n, 27), dtype=np.float32) * 0.05).astype(np.float32)
    flags[: dims[1] * dims[2]] |= SOURCE
    induced = (rng.random(27) * 1e-3).astype(np.float32)
    ref = refkern.run(dims, points_from(f, flags), "SRCF", nsteps=6, tau=0.75, tab_cells=cells, tab_records=recs,
                      flow_criterion=2, induced=induced, threads=threads)
    with lbm.Lattice(*dims, mode="d3q27_ref", tau=0.75, order=lbm.ORDER_CLI) as L:
        L.set_equilibrium_evaluation(eq)
        L.load_aos(points_from(f, flags))
        L.set_reflection_tables(cells, recs)
        L.set_flow(flags & SOURCE, induced)
        L.step(6)
        got = L.retrieve_aos()
    assert np.array_equal(got["isInternal"], ref["isInternal"])
    assert np.array_equal(got["isReflected"], ref["isReflected"])
    close(got["f"], ref["f"])
