"""Extract the reference's known answers into tests/golden/reference_known_answers.json.

Run once, where the reference sources are readable:

    python tests/golden/make_golden.py <reference checkout>

It reads the reference's GoogleTest files as text and records every EXPECT_NEAR / EXPECT_EQ /
EXPECT_TRUE / EXPECT_FALSE assertion of the tests that pin the collide-stream path, with the test
name, the source file and line, the asserted expression and the expected value, and the vertex and
face lists of the test meshes (test/dataFiles/*.obj) that those tests load.  The parity tests
(tests/test_oracle_golden.py, tests/test_gpu_d3q27_ref.py) rebuild each test's set-up and compare
against these values, so the fixture holds only numbers that the reference's own tests state.
"""
from __future__ import annotations

import json
import os
import re
import sys

FILES = ["test/CalculationsTest.cpp", "test/CoordinatesTest.cpp", "test/GeometryTest.cpp",
         "test/ModelTest.cpp"]
TEST_RE = re.compile(r"^\s*TEST\((\w+),\s*(\w+)\)")
NEAR_RE = re.compile(r"EXPECT_NEAR\((.+),\s*([-+0-9.eE]+|[\w:]+|\w+\.[xyz])\s*,\s*([-+0-9.eE]+|[\w:]+)\);")
EQ_RE = re.compile(r"EXPECT_EQ\((.+),\s*([-+0-9.eE]+|[\w.\[\]]+)\);")
BOOL_RE = re.compile(r"EXPECT_(TRUE|FALSE)\((.+)\);")
PAIR_RE = re.compile(r"std::pair<float, int>\{([-+0-9.eE]+),\s*(\d+)\}")
# 3-vectors set up by a test: `Point_3 name(a, b, c);`, `name = Point_3(a, b, c);` (also the CGAL
# point type), and the angle of a rotateVectorAroundAxis call
VEC_RE = re.compile(r"(?:Point_3\s+(\w+)\s*\(|(\w+)\s*=\s*(?:CGAL::Simple_cartesian<float>::)?Point_3\s*\()(.*)\);")
ROT_RE = re.compile(r"rotateVectorAroundAxis\((\w+),\s*(\w+),\s*(.+)\);")


def _eval(expr: str) -> float:
    """Value of a numeric C++ expression built from literals, M_PI, cos, sin and + - * /."""
    import ast
    import math
    tree = ast.parse(expr.replace("M_PI", "pi"), mode="eval")

    def ev(n):
        if isinstance(n, ast.Expression):
            return ev(n.body)
        if isinstance(n, ast.Constant) and isinstance(n.value, (int, float)):
            return float(n.value)
        if isinstance(n, ast.Name) and n.id == "pi":
            return math.pi
        if isinstance(n, ast.UnaryOp) and isinstance(n.op, ast.USub):
            return -ev(n.operand)
        if isinstance(n, ast.BinOp) and isinstance(n.op, (ast.Add, ast.Sub, ast.Mult, ast.Div)):
            a, b = ev(n.left), ev(n.right)
            return {ast.Add: a + b, ast.Sub: a - b, ast.Mult: a * b, ast.Div: a / b if b else math.nan}[type(n.op)]
        if isinstance(n, ast.Call) and isinstance(n.func, ast.Name) and n.func.id in ("cos", "sin") and len(n.args) == 1:
            return getattr(math, n.func.id)(ev(n.args[0]))
        raise ValueError(f"unsupported expression {expr!r}")
    return ev(tree)


def _split_args(text: str):
    depth, cur, out = 0, "", []
    for ch in text:
        if ch == "," and depth == 0:
            out.append(cur.strip())
            cur = ""
            continue
        depth += ch == "("
        depth -= ch == ")"
        cur += ch
    out.append(cur.strip())
    return out


def _num(tok):
    try:
        return float(tok)
    except ValueError:
        return tok


def extract(root: str) -> dict:
    out = {"source": "reference GoogleTest files, read as text", "assertions": []}
    for rel in FILES:
        path = os.path.join(root, rel)
        test = None
        with open(path) as fh:
            for lineno, line in enumerate(fh, 1):
                m = TEST_RE.match(line)
                if m:
                    test = f"{m.group(1)}.{m.group(2)}"
                    continue
                rec = None
                m = VEC_RE.search(line)
                if m and test:
                    args = _split_args(m.group(3))
                    if len(args) == 3:
                        out["assertions"].append({"test": test, "file": rel, "line": lineno, "kind": "vector",
                                                  "name": m.group(1) or m.group(2),
                                                  "value": [_eval(a) for a in args]})
                    continue
                m = ROT_RE.search(line)
                if m and test:
                    out["assertions"].append({"test": test, "file": rel, "line": lineno, "kind": "rotation",
                                              "axis": m.group(1), "vector": m.group(2),
                                              "angle": _eval(m.group(3))})
                    continue
                m = NEAR_RE.search(line)
                if m:
                    rec = {"kind": "near", "expr": m.group(1).strip(), "value": _num(m.group(2)),
                           "tol": _num(m.group(3))}
                else:
                    m = EQ_RE.search(line)
                    if m:
                        rec = {"kind": "eq", "expr": m.group(1).strip(), "value": _num(m.group(2))}
                    else:
                        m = BOOL_RE.search(line)
                        if m:
                            rec = {"kind": m.group(1).lower(), "expr": m.group(2).strip()}
                if rec is None:
                    # the distributeVector expectations live in an initialiser list
                    pairs = PAIR_RE.findall(line)
                    if pairs and "expected" in line:
                        out["assertions"].append({
                            "test": test, "file": rel, "line": lineno, "kind": "pairs",
                            "value": [[float(a), int(b)] for a, b in pairs]})
                    continue
                rec.update({"test": test, "file": rel, "line": lineno})
                out["assertions"].append(rec)
    # the named tolerance the geometry tests use (simulation/source/Constants.cpp)
    out["constants"] = {}
    with open(os.path.join(root, "simulation", "source", "Constants.cpp")) as fh:
        for line in fh:
            m = re.search(r"const float (GEOMETRIC_TOLERANCE)\s*=\s*([-+0-9.eE]+);", line)
            if m:
                out["constants"][m.group(1)] = float(m.group(2))
    out["meshes"] = {}
    meshdir = os.path.join(root, "test", "dataFiles")
    for name in sorted(os.listdir(meshdir)):
        if not name.endswith(".obj"):
            continue
        verts, faces = [], []
        with open(os.path.join(meshdir, name)) as fh:
            for line in fh:
                tok = line.split("#", 1)[0].split()
                if not tok:
                    continue
                if tok[0] == "v":
                    verts.append([float(t) for t in tok[1:4]])
                elif tok[0] == "f":
                    faces.append([int(t.split("/")[0]) - 1 for t in tok[1:]])
        out["meshes"][name] = {"file": f"test/dataFiles/{name}", "vertices": verts, "faces": faces}
    return out


def main():
    if len(sys.argv) != 2:
        sys.exit("usage: python tests/golden/make_golden.py <reference checkout>")
    root = sys.argv[1]
    data = extract(root)
    dst = os.path.join(os.path.dirname(os.path.abspath(__file__)), "reference_known_answers.json")
    with open(dst, "w") as fh:
        json.dump(data, fh, indent=1)
    print(f"wrote {len(data['assertions'])} assertions to {dst}")


if __name__ == "__main__":
    main()
