"""Checkpoint and resume (lbm_save / lbm_load / lbm_checkpoint_desc): a run interrupted by a save and
continued from the file in a new context gives, bit for bit, what the uninterrupted run gives -- D2Q9
in every storage type with walls, moving walls, periodic edges and force, and D3Q27_REF with
reflection tables, flow source and accumulated force in both fast equilibrium evaluations."""
import numpy as np
import pytest

import latticeboltzmanncuda_gb300 as lbm
from refcases import SOURCE
from test_gpu_d3q27_ref import random_lattice

pytestmark = pytest.mark.gpu


def points(f, flags):
    pts = np.zeros(f.shape[0], lbm.LATTICE_POINT)
    pts["f"] = f
    pts["isInternal"] = (flags & 1) != 0
    pts["isReflected"] = (flags & 2) != 0
    return pts


@pytest.mark.parametrize("dtype", ["f32", "f16s", "bf16s", "f64"])
def test_d2q9_resume_is_bitwise(tmp_path, dtype):
    nx, ny = 203, 77
    flags, _ = lbm.gen_channel(nx, ny, 5, 3.0, 7.0, 4)
    flags[ny // 2, ::9] = lbm.MOVING_WALL
    kw = dict(dtype=dtype, tau=0.58, periodic=1, body_force=(2e-5, 1e-6, 0), wall_velocity=(0.02, 0, 0))
    path = tmp_path / "state.lbm"
    with lbm.Lattice(nx, ny, **kw) as L:
        L.set_flags(flags)
        L.init_equilibrium()
        L.step(37)
        L.save(path)
        L.step(25)
        want = L.retrieve_populations(np.float64)
        want_steps = L.info()["steps_done"]
    with lbm.Lattice.from_checkpoint(path) as R:
        assert R.info()["steps_done"] == 37
        assert np.array_equal(R.get_flags(), flags)
        R.step(25)
        got = R.retrieve_populations(np.float64)
        assert R.info()["steps_done"] == want_steps
    assert np.array_equal(got, want)


@pytest.mark.parametrize("eq", ["float_float", "fp32"])
def test_d3q27_resume_is_bitwise(tmp_path, eq):
    dims = (12, 8, 12)
    f, flags, cells, recs, induced = random_lattice(dims, 41)
    path = tmp_path / "state.lbm"
    with lbm.Lattice(*dims, mode="d3q27_ref", tau=0.7, order=lbm.ORDER_CLI) as L:
        L.set_equilibrium_evaluation(eq)
        L.load_aos(points(f, flags))
        L.set_reflection_tables(cells, recs)
        L.set_flow(flags & SOURCE, induced)
        L.set_force((0.5, -0.25, 0.125), True)
        L.step(3)
        L.save(path)
        L.step(4)
        want, want_force = L.retrieve_populations(), L.get_force()
    with lbm.Lattice.from_checkpoint(path) as R:
        R.step(4)
        got, got_force = R.retrieve_populations(), R.get_force()
    assert np.array_equal(got, want)
    assert np.array_equal(got_force, want_force)


def test_load_rejects_other_sizes_and_corrupt_files(tmp_path):
    path = tmp_path / "state.lbm"
    with lbm.Lattice(40, 30, dtype="f32", tau=0.7) as L:
        L.step(3)
        L.save(path)
    with lbm.Lattice(41, 30, dtype="f32", tau=0.7) as other:
        with pytest.raises(lbm.LBMError):
            other.load(path)
    with lbm.Lattice(40, 30, dtype="f16s", tau=0.7) as other:
        with pytest.raises(lbm.LBMError):
            other.load(path)
    data = bytearray(path.read_bytes())
    data[-5] ^= 0x40  # one flipped bit in the populations
    bad = tmp_path / "bad.lbm"
    bad.write_bytes(bytes(data))
    with lbm.Lattice(40, 30, dtype="f32", tau=0.7) as L:
        with pytest.raises(lbm.LBMError, match="checksum"):
            L.load(bad)
        short = tmp_path / "short.lbm"
        short.write_bytes(bytes(data[: len(data) // 2]))
        with pytest.raises(lbm.LBMError, match="truncated"):
            L.load(short)
