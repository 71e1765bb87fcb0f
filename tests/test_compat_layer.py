"""The reference's C++ API on this library (latticeboltzmanncuda_gb300/compat): its own GoogleTest
cases, rewritten in tests/compat/compat_tests.cpp against the compatibility headers, checked here
against the expected values of tests/golden/; and the reference's command line
(bin/LatticeBoltzmannCuda) against the CPU oracle."""
from __future__ import annotations

import json
import os
import subprocess

import numpy as np
import pytest

import latticeboltzmanncuda_gb300 as lbm
import oracle
from conftest import known
from latticeboltzmanncuda_gb300 import build as lbm_build

HERE = os.path.dirname(os.path.abspath(__file__))


@pytest.fixture(scope="module")
def meshes(tmp_path_factory, golden):
    d = tmp_path_factory.mktemp("dataFiles")
    for name, m in golden["meshes"].items():
        lines = [f"v {x!r} {y!r} {z!r}" for x, y, z in m["vertices"]]
        lines += ["f " + " ".join(str(i + 1) for i in f) for f in m["faces"]]
        (d / name).write_text("\n".join(lines) + "\n")
    return str(d)


@pytest.fixture(scope="module")
def compat_tests(tmp_path_factory):
    lbm_build.build()
    exe = str(tmp_path_factory.mktemp("compat") / "compat_tests")
    cuda_inc, cuda_lib = lbm_build.cuda_dirs()
    cmd = ["g++", "-std=c++17", "-O1", "-ffp-contract=off", "-I", os.path.join(lbm_build.COMPAT, "include"),
           "-I", lbm_build.INCLUDE, "-I", cuda_inc, os.path.join(HERE, "compat", "compat_tests.cpp"), "-o", exe,
           "-L", lbm_build.PKG, "-llbm_compat", "-llbm_gb300", f"-Wl,-rpath,{lbm_build.PKG}",
           "-L", cuda_lib, "-lcudart", f"-Wl,-rpath,{cuda_lib}"]
    subprocess.run(cmd, check=True, capture_output=True, text=True)
    return exe


def run_records(exe, meshes, host_only):
    args = [exe, meshes] + (["--host-only"] if host_only else [])
    r = subprocess.run(args, capture_output=True, text=True, timeout=600)
    assert r.returncode == 0, r.stdout + r.stderr
    return [json.loads(line) for line in r.stdout.splitlines() if line.startswith("{")]


def expected(golden, test, line):
    """(kind, value, tol) of a reference assertion, with value expressions resolved from the
    vectors and initialiser lists the same reference test sets up."""
    if test == "CoordinatesTest.TestDistributeVector" and line in (192, 193, 194):
        # EXPECT_NEAR(result[k].first, expected[k].first, GEOMETRIC_TOLERANCE), expected from line 182
        pairs = known(golden, test, 182)["value"]
        return "near", pairs[line - 192][0], golden["constants"]["GEOMETRIC_TOLERANCE"]
    rec = known(golden, test, line)
    kind, value, tol = rec["kind"], rec.get("value"), rec.get("tol")
    if isinstance(tol, str):
        tol = golden["constants"][tol.split("::")[-1]]
    if isinstance(value, str):
        if value.startswith("expected[") and value.endswith("].second"):
            value = known(golden, test, 182)["value"][int(value[9])][1]
        elif "." in value:
            name, comp = value.split(".")
            vecs = [a for a in golden["assertions"] if a["test"] == test and a.get("kind") == "vector"
                    and a["name"] == name and a["line"] < line]
            value = max(vecs, key=lambda a: a["line"])["value"]["xyz".index(comp)]
        elif value == "value":  # EXPECT_EQ(result, value): the program reports the comparison
            kind, value = "true", None
    return kind, value, tol


def check_records(golden, records, minimum):
    assert len(records) >= minimum
    for r in records:
        kind, value, tol = expected(golden, r["test"], r["line"])
        if "mismatches" in r:
            assert r["mismatches"] == 0, r
        elif kind == "near":
            assert abs(r["got"] - value) <= tol, (r, value, tol)
        elif kind == "eq":
            assert r["got"] == value, (r, value)
        elif kind == "true":
            assert r["got"] == 1, r
        elif kind == "false":
            assert r["got"] == 0, r
        else:
            raise AssertionError(f"unhandled assertion kind {kind} for {r}")


def test_compat_headers_and_host_cases(golden, compat_tests, meshes):
    """ModelTest, GeometryTest, CompressionTest and TestDistributeVector through the reference's C++
    API; they need no GPU."""
    records = run_records(compat_tests, meshes, host_only=True)
    check_records(golden, records, minimum=22)
    tests = {r["test"] for r in records}
    assert {"ModelTest.intersectionNormal", "GeometryTest.TestQuaternionRoatation",
            "CalculationsTest.CompressionTest", "CoordinatesTest.TestDistributeVector"} <= tests


@pytest.mark.gpu
def test_compat_all_reference_cases(golden, compat_tests, meshes):
    """Every reference test case that exercises the collide-stream path, through the C++ API."""
    records = run_records(compat_tests, meshes, host_only=False)
    check_records(golden, records, minimum=60)
    tests = {r["test"] for r in records}
    # TestReflectionsData runs twice: host ReflectionData through Lattice, device ReflectionData
    # (cudaMalloc, as Lattice.cpp:58 makes it) through RunCudaFunctions::run_calculate_reflections_data
    assert sum(r["test"] == "CalculationsTest.TestReflectionsData" and r["line"] == 194 for r in records) == 2
    for t in ("CalculationsTest.TestStreaming", "CalculationsTest.TestCollision", "CalculationsTest.TestFull",
              "CalculationsTest.TestReflections", "CalculationsTest.TestReflectionsData",
              "CalculationsTest.TestFlowGeneration", "CalculationsTest.TestPlaneFlowGeneration",
              "CoordinatesTest.TestCoordsMatch", "CoordinatesTest.TestCoordinatesWithModel",
              "CoordinatesTest.TestReflection"):
        assert t in tests, t


# ------------------------------------------------------------------ command line
def test_cli_usage():
    lbm_build.build()
    r = subprocess.run([lbm_build.CLI], capture_output=True, text=True)
    assert r.returncode != 0 and "usage" in r.stderr


def cli_reference_run(golden, dims, spacing, tau, steps):
    """The CLI's set-up and loop (LatticeBoltzmannCuda.cpp:18-93) on the CPU oracle: returns the
    force printed before every step."""
    from test_mesh_front_end import golden_mesh
    m = golden_mesh(golden, "compat_cube.obj")
    flags, _ = m.rasterize(dims, spacing)
    cells, recs, flags = m.reflection_tables(dims, spacing, flags)
    X, Y, Z = dims
    n = X * Y * Z
    flow = np.full(27, 0.001, np.float32)
    flow[6] = 0.002
    f = np.tile(flow, (n, 1))
    flags = flags.copy()
    flags[: Y * Z] |= 4  # FlowCriterion::testPlaneCriteria: x == 0
    tab_idx = np.full(n, -1, np.int32)
    tab_idx[cells] = np.arange(len(cells), dtype=np.int32)
    force = np.zeros(3, np.float32)
    out = [force.copy()]
    for _ in range(steps - 1):
        f = oracle.d3q27_run(dims, f, flags, tau, 1, order=1, tab_idx=tab_idx, tabs=recs, induced=flow, force=force,
                             force_mode=0)
        out.append(force.copy())
    return np.array(out)


@pytest.mark.gpu
def test_cli_matches_oracle(golden, meshes):
    """The reference's command line on compat_cube (10^3 cells, spacing 0.1): the printed force
    series equals the oracle's within the print precision (6 significant digits) and 1e-5."""
    lbm_build.build()
    steps = 12
    args = [lbm_build.CLI, os.path.join(meshes, "compat_cube.obj"), "2", "5", "1", "5", "2", "10", "1.0", "0.9", "0.1",
            str(steps)]
    r = subprocess.run(args, capture_output=True, text=True, timeout=300)
    assert r.returncode == 0, r.stdout + r.stderr
    lines = [l for l in r.stdout.splitlines() if l.strip()]
    assert len(lines) == steps
    got = np.array([[float(v) for v in l.split()] for l in lines])
    want = cli_reference_run(golden, (10, 10, 10), 0.1, 0.9, steps)
    scale = max(1e-30, float(np.max(np.abs(want))))
    assert np.all(np.abs(got - want) <= 1e-5 * scale + 5e-6 * np.abs(want)), (got, want)
    assert np.any(np.abs(want[-1]) > 0)
