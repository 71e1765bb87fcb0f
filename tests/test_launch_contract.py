"""CPU check of the programmatic dependent launch contract (csrc/pdl.cuh) on the kernel sources.

A kernel launched through launch_maybe_dependent may start while the grid before it in the stream
is still running, so every path of it must execute wait_prerequisite_grids() before it loads or
stores anything that grid reads or writes.  The contract per kernel:

* the D2Q9 vector step and the four batch step kernels: the wait is the first statement of the
  kernel, before any early return, and allow_dependent_launch() follows it;
* the D3Q27 gather kernel (the programmatic dependent of the previous step's fused kernel): the
  wait is its first statement;
* the D3Q27 fused kernel: the wait precedes the read of a gathered row (the only data the gather
  grid before it writes), and one thread of the last block waits unconditionally, so the fused
  grid never completes before the gather grid; the gather kernel allows its launch only after its
  own wait, so the fused kernel starts after the previous step's fused kernel has completed;
* every kernel named in a launch_maybe_dependent call is one of those above.
"""
import os
import re

import pytest

CSRC = os.path.join(os.path.dirname(os.path.dirname(os.path.abspath(__file__))), "latticeboltzmanncuda_gb300", "csrc")


def source(name):
    with open(os.path.join(CSRC, name)) as fh:
        return fh.read()


def kernel_body(src, name):
    """The text of the first `__global__` function called `name` between its braces."""
    m = re.search(r"__global__[^{;]*?\b" + re.escape(name) + r"\s*\(", src)
    assert m, f"kernel {name} not found"
    i = src.index("{", m.end())
    depth = 0
    for j in range(i, len(src)):
        depth += {"{": 1, "}": -1}.get(src[j], 0)
        if depth == 0:
            return src[i + 1:j]
    raise AssertionError(f"unbalanced braces in {name}")


def statements(body):
    """Statements of a body without comments, blank lines and preprocessor lines."""
    body = re.sub(r"//[^\n]*", "", body)
    return [s.strip() for s in body.split(";") if s.strip()]


def launched_dependent(src):
    """Kernel names passed to launch_maybe_dependent (template arguments stripped)."""
    return {re.sub(r"<.*", "", m) for m in re.findall(r"launch_maybe_dependent\(\s*[^,]+,\s*([A-Za-z_][\w:]*(?:<[^>]*>)?)", src)}


WAIT_FIRST = {
    "d2q9.cu": {"step_vec_kernel"},
    "batch.cu": {"batch_step_kernel", "batch_step_kernel_occ", "batch_step_kernel_p", "batch_step_kernel_p_occ"},
}


@pytest.mark.parametrize("fname", sorted(WAIT_FIRST))
def test_dependent_kernels_wait_first(fname):
    src = source(fname)
    for name in WAIT_FIRST[fname]:
        st = statements(kernel_body(src, name))
        assert st[0] == "wait_prerequisite_grids()", (name, st[:2])
        assert st[1] == "allow_dependent_launch()", (name, st[:2])


@pytest.mark.parametrize("fname", ["d2q9.cu", "batch.cu", "d3q27.cu"])
def test_only_contracted_kernels_are_launched_as_dependents(fname):
    src = source(fname)
    allowed = WAIT_FIRST.get(fname, set()) | ({"fused_kernel", "gather_kernel"} if fname == "d3q27.cu" else set())
    launched = launched_dependent(src)
    assert launched, f"no dependent launch found in {fname}"
    assert launched <= allowed, launched - allowed


def test_fused_kernel_waits_before_reading_gathered_rows():
    src = source("d3q27.cu")
    cell = src[src.index("__device__ __forceinline__ bool fused_cell("):]
    cell = cell[:cell.index("\n}\n")]
    branch = cell[cell.index("if (a.cli && (fl & F_GATHER))"):]
    assert branch.index("wait_prerequisite_grids()") < branch.index("a.gathered"), "gathered row read before the wait"
    # the row is read through L2, not the read-only path
    assert "__ldg(g + j)" not in branch and "__ldcg(g + j)" in branch
    body = statements(kernel_body(src, "fused_kernel"))
    assert body[0] == "if (blockIdx.x == gridDim.x - 1 && threadIdx.x == 0) wait_prerequisite_grids()", body[0]
    # the gather kernel waits first, then allows the launch of its dependent
    gather = statements(kernel_body(src, "gather_kernel"))
    assert gather[0] == "wait_prerequisite_grids()", gather[0]
    assert gather[1] == "if (MODE == 0) allow_dependent_launch()", gather[1]
    assert "allow_dependent_launch()" in body[1], body[1]


def test_contract_check_catches_a_load_before_the_wait():
    """The statement check rejects a kernel whose first statement is not the wait."""
    bad = "__global__ void k(const float *p, float *q) {\n    q[0] = p[0];\n    wait_prerequisite_grids();\n}\n"
    st = statements(kernel_body(bad, "k"))
    assert st[0] != "wait_prerequisite_grids()"
