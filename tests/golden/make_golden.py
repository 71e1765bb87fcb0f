"""Extract the reference's known answers into tests/golden/reference_known_answers.json.

Run once, where the reference sources are readable:

    python tests/golden/make_golden.py /root/reference

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
NEAR_RE = re.compile(r"EXPECT_NEAR\((.+),\s*([-+0-9.eE]+|[\w:]+)\s*,\s*([-+0-9.eE]+|[\w:]+)\);")
EQ_RE = re.compile(r"EXPECT_EQ\((.+),\s*([-+0-9.eE]+|[\w.\[\]]+)\);")
BOOL_RE = re.compile(r"EXPECT_(TRUE|FALSE)\((.+)\);")
PAIR_RE = re.compile(r"std::pair<float, int>\{([-+0-9.eE]+),\s*(\d+)\}")


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
    root = sys.argv[1] if len(sys.argv) > 1 else "/root/reference"
    data = extract(root)
    dst = os.path.join(os.path.dirname(os.path.abspath(__file__)), "reference_known_answers.json")
    with open(dst, "w") as fh:
        json.dump(data, fh, indent=1)
    print(f"wrote {len(data['assertions'])} assertions to {dst}")


if __name__ == "__main__":
    main()
