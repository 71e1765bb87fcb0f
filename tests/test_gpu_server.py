"""The continuous-batching server (lbm_server_run): every request's result is bit-identical to the
same solve run alone, admission follows the memory budget and the slot limit, and failures are
per-request (over-budget, invalid input) or bounded (time limit) -- all made on the host."""
from dataclasses import dataclass

import numpy as np
import pytest

import latticeboltzmanncuda_gb300 as lbm
from latticeboltzmanncuda_gb300 import capi

pytestmark = pytest.mark.gpu


@dataclass
class Req:
    nx: int
    ny: int
    tau: float
    flags: np.ndarray
    periodic: int
    body_force: tuple
    wall_velocity: tuple
    steps: int
    arrival: float


def make_requests(n, seed=5):
    rng = np.random.default_rng(seed)
    out = []
    for i in range(n):
        nx, ny = int(rng.integers(24, 140)), int(rng.integers(16, 90))
        if i % 2:
            fl = lbm.gen_cavity(nx, ny)
            per, force, wall = 0, (0.0, 0.0), (0.04, 0.0)
        else:
            fl = np.zeros((ny, nx), np.uint8)
            fl[0, :] = fl[-1, :] = 1
            per, force, wall = 1, (2e-6, 0.0), (0.0, 0.0)
        fl, _ = lbm.gen_disks_fraction(fl, float(rng.uniform(0, 0.2)), 1.5, 4.0, 100 + i)
        out.append(Req(nx, ny, float(rng.uniform(0.55, 1.1)), fl, per, force, wall, int(rng.integers(50, 400)),
                       float(0.0002 * i)))
    return out


def solo(r, dtype):
    with lbm.Lattice(r.nx, r.ny, dtype=dtype, tau=r.tau, periodic=r.periodic, body_force=(*r.body_force, 0),
                     wall_velocity=(*r.wall_velocity, 0)) as L:
        L.set_flags(r.flags)
        L.init_equilibrium()
        L.step(r.steps)
        return L.moments()


@pytest.mark.parametrize("dtype", ["f32", "f16s"])
def test_results_equal_solo_runs(dtype):
    reqs = make_requests(10)
    results, stats, status = lbm.serve(reqs, dtype=dtype, round_steps=64, outputs=True)
    assert status == capi.OK
    assert stats["peak_slots"] > 1  # requests did overlap
    assert stats["cell_updates"] == sum(r.nx * r.ny * r.steps for r in reqs)
    for r, res in zip(reqs, results):
        assert res["status"] == capi.OK
        assert res["admitted"] >= r.arrival - 1e-6 and res["finished"] >= res["admitted"]
        for got, want in zip(res["moments"], solo(r, dtype)):
            assert np.array_equal(got, want)


def test_budget_limits_live_solves():
    reqs = make_requests(8)
    per_slot = max(lbm.Batch.slot_bytes("f32", r.nx, r.ny) for r in reqs)
    results, stats, status = lbm.serve(reqs, budget_bytes=2 * per_slot, round_steps=50)
    assert status == capi.OK
    assert all(r["status"] == capi.OK for r in results)
    assert stats["peak_bytes"] <= 2 * per_slot  # the budget bounds the bytes, not the count
    assert stats["peak_slots"] >= 2


def test_slot_limit_serialises():
    """With one slot the solves run one after another in arrival order: a request is admitted
    once the previous one has been retired (its read-back and free queued behind its last round,
    so the device never holds two), and they complete in the same order, each equal to its solo
    run."""
    reqs = make_requests(5)
    results, stats, status = lbm.serve(reqs, max_slots=1, round_steps=1000, outputs=True)
    assert status == capi.OK and stats["peak_slots"] == 1
    by_arrival = sorted(range(len(reqs)), key=lambda i: reqs[i].arrival)
    adm = [results[i]["admitted"] for i in by_arrival]
    fin = [results[i]["finished"] for i in by_arrival]
    assert adm == sorted(adm) and fin == sorted(fin)
    assert all(a <= f for a, f in zip(adm, fin))
    for i in by_arrival:
        for got, want in zip(results[i]["moments"], solo(reqs[i], "f32")):
            assert np.array_equal(got, want)


def test_over_budget_and_invalid_requests_fail_alone():
    reqs = make_requests(4)
    big = Req(4096, 4096, 0.6, None, 0, (0.0, 0.0), (0.0, 0.0), 10, 0.0)
    bad_flags = np.full((20, 20), 9, np.uint8)
    bad = Req(20, 20, 0.6, bad_flags, 0, (0.0, 0.0), (0.0, 0.0), 10, 0.001)
    budget = 4 * max(lbm.Batch.slot_bytes("f32", r.nx, r.ny) for r in reqs)
    results, stats, status = lbm.serve(reqs + [big, bad], budget_bytes=budget, round_steps=50)
    assert status == capi.OK
    assert [r["status"] for r in results[:4]] == [capi.OK] * 4
    assert results[4]["status"] == capi.ERR_BUDGET and stats["rejected"] == 1
    assert results[5]["status"] == capi.ERR_INVALID


def test_time_limit_ends_the_run():
    reqs = make_requests(3)
    for r in reqs:
        r.steps = 10_000_000  # far more than the limit allows
    results, stats, status = lbm.serve(reqs, round_steps=20, time_limit=0.3)
    assert status == capi.ERR_TIMEOUT
    assert all(r["status"] == capi.ERR_TIMEOUT for r in results)
    assert stats["makespan"] < 5.0
