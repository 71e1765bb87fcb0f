"""Mesh front end (lbm_mesh_*, csrc/mesh.cpp) against the reference's own known answers:
test/ModelTest.cpp, test/GeometryTest.cpp, test/CoordinatesTest.cpp:137-229, and -- through the
CPU oracle's reflection pass -- test/CalculationsTest.cpp:107-197 with tables built from the mesh
instead of injected.  Host code only: no GPU needed."""
from __future__ import annotations

import math

import numpy as np
import pytest

import latticeboltzmanncuda_gb300 as lbm
import oracle
from conftest import known
from refcases import INTERNAL, REFLECTED, cell, icosphere


def golden_mesh(golden, name):
    m = golden["meshes"][name]
    return lbm.Mesh.from_arrays(m["vertices"], m["faces"])


def write_obj(path, golden, name, style=0):
    """Write a golden mesh as OBJ text; style varies the record forms the reader must accept."""
    m = golden["meshes"][name]
    lines = ["# written by the test", "o model"]
    lines += [f"v {x!r} {y!r} {z!r}" for x, y, z in m["vertices"]]
    lines += ["vn 0 0 1", "vt 0 0"]
    nv = len(m["vertices"])
    for f in m["faces"]:
        if style == 0:
            toks = [str(i + 1) for i in f]
        elif style == 1:
            toks = [f"{i + 1}/1/1" for i in f]
        else:
            toks = [f"{i - nv}//1" for i in f]  # negative (relative) indices
        lines.append("f " + " ".join(toks) + "   # face")
    path.write_text("\n".join(lines) + "\n")
    return str(path)


def vec(golden, test, line):
    return known(golden, test, line)["value"]


# ---------------------------------------------------------------- test/ModelTest.cpp

@pytest.mark.parametrize("style", [0, 1, 2])
def test_import_model(golden, tmp_path, style):
    # ModelTest.cpp:5-12
    with lbm.Mesh.load_obj(write_obj(tmp_path / "t.obj", golden, "triangle.obj", style)) as m:
        assert m.info()["vertices"] == known(golden, "ModelTest.importModel", 11)["value"]
    with lbm.Mesh.load_obj(write_obj(tmp_path / "c.obj", golden, "cube_angled.obj", style)) as m, \
            golden_mesh(golden, "cube_angled.obj") as g:
        assert m.info() == g.info()
        assert np.array_equal(m.reflection_vector((1.0, 0.5, 0.5), (0.5, 0.5, 0.5)),
                              g.reflection_vector((1.0, 0.5, 0.5), (0.5, 0.5, 0.5)))


def test_model_closed(golden):
    # ModelTest.cpp:14-25
    assert known(golden, "ModelTest.isModelClosed", 20)["kind"] == "true"
    assert golden_mesh(golden, "cube.obj").info()["closed"]
    assert known(golden, "ModelTest.isModelClosed", 24)["kind"] == "false"
    assert not golden_mesh(golden, "triangle.obj").info()["closed"]


def test_point_inside_model(golden):
    # ModelTest.cpp:27-40
    m = golden_mesh(golden, "cube.obj")
    assert m.point_inside(vec(golden, "ModelTest.isPointInsideModel", 33))
    assert not m.point_inside(vec(golden, "ModelTest.isPointInsideModel", 37))


def test_check_error_model(golden):
    # ModelTest.cpp:42-49: a quad face is not a triangle mesh
    assert known(golden, "ModelTest.checkErrorModel", 48)["kind"] == "true"
    for name in ("quad.obj", "quad_angled.obj", "triangle.obj"):
        info = golden_mesh(golden, name).info()
        assert not info["valid"], name
        assert not golden_mesh(golden, name).point_inside((0.5, 0.5, 0.1))


def test_intersection_normal(golden):
    # ModelTest.cpp:51-74
    t = "ModelTest.intersectionNormal"
    m = golden_mesh(golden, "compat_cube.obj")
    r = m.reflection_vector(vec(golden, t, 57), vec(golden, t, 58))
    want = vec(golden, t, 61)
    for k, line in enumerate((63, 64, 65)):
        assert abs(float(r[k]) - want[k]) <= known(golden, t, line)["tol"]
    r = m.reflection_vector(vec(golden, t, 57), vec(golden, t, 67))
    assert known(golden, t, 73)["kind"] == "eq"
    assert list(r) == vec(golden, t, 71)  # exact: no face is hit


# ---------------------------------------------------------------- test/GeometryTest.cpp

def test_quaternion_rotation(golden):
    # GeometryTest.cpp:11-32
    t = "GeometryTest.TestQuaternionRoatation"
    tol = golden["constants"]["GEOMETRIC_TOLERANCE"]
    axis, v = vec(golden, t, 13), vec(golden, t, 15)
    for rot_line, exp_line, near_lines in ((19, 17, (21, 22, 23)), (27, 25, (29, 30, 31))):
        rot = known(golden, t, rot_line)
        assert rot["axis"] == "axis" and rot["vector"] == "vector"
        got = lbm.rotate_vector(axis, v, rot["angle"])
        want = vec(golden, t, exp_line)
        for k, line in enumerate(near_lines):
            assert known(golden, t, line)["kind"] == "near"
            assert abs(float(got[k]) - want[k]) <= tol, (rot_line, k, got, want)


def test_rotation_by_pi_is_a_reflection():
    """A rotation by pi about n maps v to 2 (v.n) n - v (the reflection the mesh front end uses)."""
    rng = np.random.default_rng(3)
    for _ in range(200):
        n = rng.standard_normal(3)
        n /= np.linalg.norm(n)
        v = rng.standard_normal(3)
        got = lbm.rotate_vector(n, v, math.pi)
        assert np.allclose(got, 2 * np.dot(v, n) * n - v, atol=2e-6 * (1 + np.linalg.norm(v)))


# ---------------------------------------------------------------- test/CoordinatesTest.cpp

def test_distribute_vector(golden):
    # CoordinatesTest.cpp:171-198
    t = "CoordinatesTest.TestDistributeVector"
    tol = golden["constants"]["GEOMETRIC_TOLERANCE"]
    score, dirs = lbm.distribute_vector(vec(golden, t, 180))
    top = score[:3] / score[:3].sum()
    for k, (w, d) in enumerate(known(golden, t, 182)["value"]):
        assert abs(float(top[k]) - w) <= tol
        assert int(dirs[k]) == d


def test_distribute_vector_order():
    """Scores descend; equal scores list the larger direction first (a max-heap of (score, q))."""
    rng = np.random.default_rng(5)
    for v in [rng.standard_normal(3) for _ in range(50)] + [(1, 0, 0), (0, 0, 0), (1, 1, 0)]:
        score, dirs = lbm.distribute_vector(v)
        assert sorted(dirs.tolist()) == list(range(27))
        for i in range(26):
            assert score[i] > score[i + 1] or (score[i] == score[i + 1] and dirs[i] > dirs[i + 1])


def test_coordinates_with_model(golden):
    # CoordinatesTest.cpp:137-169: 10^3 lattice, spacing 0.1, compat_cube
    m = golden_mesh(golden, "compat_cube.obj")
    flags, applied = m.rasterize((10, 10, 10), 0.1)
    assert applied
    t = "CoordinatesTest.TestCoordinatesWithModel"
    assert known(golden, t, 158)["kind"] == "false" and known(golden, t, 166)["kind"] == "true"
    for y in range(10):
        for x in range(10):
            assert not flags[(10 * y) + x] & INTERNAL
    for y in range(1, 9):
        for x in range(1, 9):
            assert flags[500 + (10 * y) + x] & INTERNAL


def test_rasterize_keeps_flags_when_model_does_not_fit(golden):
    """insertModel returns without changes when the model's box leaves the lattice (Lattice.cpp:236-244)."""
    m = golden_mesh(golden, "cube.obj")  # spans [-1, 1]^3
    before = np.full(27, REFLECTED, np.uint8)
    after, applied = m.rasterize((3, 3, 3), 0.5, before)
    assert not applied and np.array_equal(after, before)


def test_reflection_table(golden):
    # CoordinatesTest.cpp:200-229: cell 13 of the 3^3 lattice at spacing 0.5, cube_angled
    t = "CoordinatesTest.TestReflection"
    m = golden_mesh(golden, "cube_angled.obj")
    flags, applied = m.rasterize((3, 3, 3), 0.5)
    assert applied and np.nonzero(flags & INTERNAL)[0].tolist() == [13]
    cells, recs, flags = m.reflection_tables((3, 3, 3), 0.5, flags)
    assert cells.tolist() == [13] and flags[13] & REFLECTED
    for slot, line in ((3, 223), (4, 224), (5, 225)):
        rec = known(golden, t, line)
        assert abs(float(recs[0]["w"][slot]) - rec["value"]) <= rec["tol"], (slot, recs[0]["w"][slot])
    for slot, line in ((3, 226), (4, 227), (5, 228)):
        assert oracle.refl_get_dir(recs[0], slot) == int(known(golden, t, line)["value"])


def test_reflection_table_structure(golden):
    """Every used slot group of a table holds up to 3 directions to non-internal neighbours with
    weights that sum to 1; unused groups are empty."""
    m = golden_mesh(golden, "cube_angled.obj")
    dims = (9, 9, 9)
    flags, applied = m.rasterize(dims, 0.125)
    assert applied
    cells, recs, flags = m.reflection_tables(dims, 0.125, flags)
    assert len(cells) > 0 and np.all(np.diff(cells) > 0)
    X, Y, Z = dims
    for c, r in zip(cells, recs):
        x, y, z = c // (Y * Z), (c // Z) % Y, c % Z
        assert flags[c] & INTERNAL and flags[c] & REFLECTED
        for p in range(27):
            ds = [oracle.refl_get_dir(r, 3 * p + k) for k in range(3)]
            ws = r["w"][3 * p:3 * p + 3]
            used = [d for d in ds if d]
            if not used:
                assert np.all(ws == 0)
                continue
            assert abs(float(ws[:len(used)].sum()) - 1.0) < 1e-5
            for d in used:
                nb = cell(dims, x + oracle.C27[d][0], y + oracle.C27[d][1], z + oracle.C27[d][2])
                assert not flags[nb] & INTERNAL


def test_point_in_sphere_mesh_matches_geometry():
    """Ray parity on a closed icosphere agrees with the analytic inside test away from the surface
    (the polyhedron lies between the inscribed and the circumscribed sphere)."""
    verts, faces = icosphere(3, 0.37, (0.5, 0.5, 0.5))
    m = lbm.Mesh.from_arrays(verts, faces)
    info = m.info()
    assert info["valid"] and info["faces"] == 1280
    flags, applied = m.rasterize((24, 24, 24), 1 / 23)
    assert applied
    g = np.arange(24, dtype=np.float32) * np.float32(1 / 23)
    X, Y, Z = np.meshgrid(g, g, g, indexing="ij")
    d = np.sqrt((X - 0.5) ** 2 + (Y - 0.5) ** 2 + (Z - 0.5) ** 2).reshape(-1)
    inside = (flags & INTERNAL) != 0
    assert np.all(inside[d < 0.37 * 0.985]) and not np.any(inside[d > 0.37 * 1.001])
    # reflection vectors of rays towards the centre point back outwards (the normal is radial)
    for p in ([0.95, 0.5, 0.5], [0.5, 0.05, 0.5], [0.8, 0.8, 0.8]):
        r = m.reflection_vector(p, (0.5, 0.5, 0.5))
        out = np.array(p) - 0.5
        assert np.dot(r, out / np.linalg.norm(out)) > 0.95


def test_bad_meshes_fail_loudly(tmp_path):
    with pytest.raises(lbm.LBMError):
        lbm.Mesh.load_obj(str(tmp_path / "missing.obj"))
    bad = tmp_path / "bad.obj"
    bad.write_text("v 0 0 0\nv 1 0 0\nv 0 1 0\nf 1 2 7\n")
    with pytest.raises(lbm.LBMError):
        lbm.Mesh.load_obj(str(bad))
    with pytest.raises(lbm.LBMError):
        lbm.Mesh.from_arrays([[0, 0, 0], [1, 0, 0]], [[0, 1]])
    m = lbm.Mesh.from_arrays([[0, 0, 0], [1, 0, 0], [0, 1, 0]], [[0, 1, 2]])
    with pytest.raises(lbm.LBMError):
        m.rasterize((0, 3, 3), 0.5)


# ------------------------------------------- test/CalculationsTest.cpp through the CPU oracle

@pytest.mark.parametrize("with_force", [False, True])
def test_reflections_from_mesh_tables(golden, with_force):
    """CalculationsTest.cpp:107-197 end to end on the host: insertModel + preProcessModel by the
    mesh front end, then the oracle's reflection pass (SimCalcFuncs.cu:158-198)."""
    dims = (3, 3, 3)
    m = golden_mesh(golden, "cube_angled.obj")
    flags, _ = m.rasterize(dims, 0.5)
    cells, recs, flags = m.reflection_tables(dims, 0.5, flags)
    f = np.zeros((27, 27), np.float32)
    f[cell(dims, 1, 1, 1), 1] = 1.0
    tab_idx = np.full(27, -1, np.int32)
    tab_idx[cells] = np.arange(len(cells), dtype=np.int32)
    force = np.zeros(3, np.float32) if with_force else None
    out = oracle.d3q27_reflect(dims, f, flags, tab_idx, recs, force=force, force_mode=0)
    name = "CalculationsTest.TestReflectionsData" if with_force else "CalculationsTest.TestReflections"
    lines = (186, 187, 188, 190) if with_force else (141, 142, 143, 145)
    for (x, y, z, q), line in zip(((2, 1, 2, 17), (1, 1, 2, 4), (2, 2, 2, 26), (1, 1, 1, 1)), lines):
        rec = known(golden, name, line)
        assert abs(float(out[cell(dims, x, y, z), q]) - rec["value"]) <= rec["tol"], (line, out[cell(dims, x, y, z), q])
    if with_force:
        for k, line in enumerate((194, 195, 196)):
            rec = known(golden, "CalculationsTest.TestReflectionsData", line)
            assert abs(float(force[k]) - rec["value"]) <= rec["tol"], (k, force[k], rec["value"])
