"""Batched domains (lbm_batch_*): every slot computes exactly what a single-domain context computes
(bit-identical populations), alone or in any mix, with slots joining and leaving between steps;
FP64 slots match the CPU oracle to 1e-12."""
import numpy as np
import pytest

import latticeboltzmanncuda_gb300 as lbm
import oracle

pytestmark = pytest.mark.gpu


def box(nx, ny, lid=False):
    fl = np.zeros((ny, nx), np.uint8)
    fl[0, :] = fl[:, 0] = fl[:, -1] = 1
    fl[-1, :] = 2 if lid else 1
    return fl


def specs():
    """(nx, ny, tau, flags, periodic, force, wall) for domains of uneven size and kind"""
    ch, _ = lbm.gen_channel(150, 41, 3, 2.0, 5.0, 1)
    big, _ = lbm.gen_channel(1024, 64, 6, 3.0, 8.0, 2)
    sy = np.zeros((200, 33), np.uint8)
    sy[:, 0] = 1
    sy[:, -1] = 2
    return [
        (40, 33, 0.6, box(40, 33, True), 0, (0.0, 0.0), (0.05, 0.0)),
        (150, 41, 0.55, ch, 1, (1e-5, 0.0), (0.0, 0.0)),
        (64, 64, 0.9, np.zeros((64, 64), np.uint8), 3, (0.0, 2e-6), (0.0, 0.0)),
        (97, 13, 0.7, np.zeros((13, 97), np.uint8), 0, (0.0, 0.0), (0.0, 0.0)),
        (1024, 64, 0.52, big, 1, (1e-6, 0.0), (0.0, 0.0)),
        (33, 200, 1.2, sy, 2, (0.0, 0.0), (0.02, 0.01)),
    ]


def init_state(nx, ny, seed):
    rng = np.random.default_rng(seed)
    return oracle.d2q9_equilibrium(1 + 0.01 * rng.standard_normal((ny, nx)), 0.02 * rng.standard_normal((ny, nx)),
                                   0.02 * rng.standard_normal((ny, nx)))


def single(spec, f0, steps, dtype):
    nx, ny, tau, fl, per, force, wall = spec
    with lbm.Lattice(nx, ny, dtype=dtype, tau=tau, periodic=per, body_force=(*force, 0), wall_velocity=(*wall, 0)) as L:
        L.set_flags(fl)
        L.load_populations(f0)
        L.step(steps)
        return L.retrieve_populations(np.float64)


@pytest.mark.parametrize("dtype", ["f32", "f16s", "bf16s", "f64"])
def test_batch_slots_equal_single_domains(dtype):
    sp = specs()
    steps = 37
    with lbm.Batch(dtype) as B:
        slots = []
        for i, s in enumerate(sp):
            nx, ny, tau, fl, per, force, wall = s
            slot = B.add(nx, ny, tau, fl, per, force, wall)
            B.load_populations(slot, init_state(nx, ny, i))
            slots.append(slot)
        B.step(steps)
        info = B.info()
        assert info["slots"] == len(sp) and info["tiles"] > 0
        for i, (s, slot) in enumerate(zip(sp, slots)):
            got = B.retrieve_populations(slot, np.float64)
            want = single(s, init_state(s[0], s[1], i), steps, dtype)
            assert np.array_equal(got, want), (dtype, i)
            assert B.steps_done(slot) == steps


def test_batch_fp64_matches_oracle():
    sp = specs()[:4]
    steps = 25
    with lbm.Batch("f64") as B:
        for i, (nx, ny, tau, fl, per, force, wall) in enumerate(sp):
            slot = B.add(nx, ny, tau, fl, per, force, wall)
            f0 = init_state(nx, ny, 10 + i)
            B.load_populations(slot, f0)
            # the library takes tau, force and wall velocity as float: the oracle gets the same values
            tau32, force32, wall32 = float(np.float32(tau)), tuple(float(np.float32(v)) for v in force), \
                tuple(float(np.float32(v)) for v in wall)
            ref = oracle.d2q9_run(f0, fl, tau32, steps, periodic=per, force=force32, wall_velocity=wall32)
            B.step(steps)  # one live slot at a time
            got = B.retrieve_populations(slot, np.float64)
            fluid = fl == 0
            assert np.max(np.abs(got - ref)[:, fluid]) <= 1e-12, i
            B.remove(slot)


def test_slots_join_and_leave_without_disturbing_others():
    sp = specs()
    a, b, c = sp[0], sp[1], sp[4]
    with lbm.Batch("f32") as B:
        sa = B.add(*a[:4], a[4], a[5], a[6])
        B.load_populations(sa, init_state(a[0], a[1], 0))
        sb = B.add(*b[:4], b[4], b[5], b[6])
        B.load_populations(sb, init_state(b[0], b[1], 1))
        B.step(10)
        sc = B.add(*c[:4], c[4], c[5], c[6])
        B.load_populations(sc, init_state(c[0], c[1], 4))
        B.step(7)
        ga = B.retrieve_populations(sa, np.float64)
        B.remove(sa)
        B.step(5)
        gb = B.retrieve_populations(sb, np.float64)
        gc = B.retrieve_populations(sc, np.float64)
        assert B.info()["slots"] == 2
    assert np.array_equal(ga, single(a, init_state(a[0], a[1], 0), 17, "f32"))
    assert np.array_equal(gb, single(b, init_state(b[0], b[1], 1), 22, "f32"))
    assert np.array_equal(gc, single(c, init_state(c[0], c[1], 4), 12, "f32"))


def test_step_budgets_stop_slots_mid_sequence():
    """A slot with a step budget stops when it runs out, inside one lbm_batch_step call, and its
    populations equal a solo run of exactly that many steps; slots without a budget run on."""
    sp = specs()
    budgets = [5, 12, -1, 0, 7, 30]
    with lbm.Batch("f32") as B:
        slots = []
        for i, s in enumerate(sp):
            slot = B.add(*s[:4], s[4], s[5], s[6])
            B.load_populations(slot, init_state(s[0], s[1], 40 + i))
            B.set_slot_steps(slot, budgets[i])
            slots.append(slot)
        B.step(9)
        B.step(8)
        for i, (s, slot) in enumerate(zip(sp, slots)):
            want_steps = 17 if budgets[i] < 0 else min(17, budgets[i])
            assert B.steps_done(slot) == want_steps
            got = B.retrieve_populations(slot, np.float64)
            assert np.array_equal(got, single(s, init_state(s[0], s[1], 40 + i), want_steps, "f32")), i


@pytest.mark.parametrize("shape", [(2, 32, 1), (4, 32, 4), (4, 64, 2), (4, 128, 1), (8, 32, 8)])
def test_every_batch_tile_shape(shape):
    sp = specs()
    dtype = "f16s" if shape[0] == 8 else "f32"
    with lbm.Batch(dtype) as B:
        B.set_launch(*shape)
        slots = [B.add(*s[:4], s[4], s[5], s[6]) for s in sp]
        for i, slot in enumerate(slots):
            B.load_populations(slot, init_state(sp[i][0], sp[i][1], 20 + i))
        B.step(11)
        for i, slot in enumerate(slots):
            want = single(sp[i], init_state(sp[i][0], sp[i][1], 20 + i), 11, dtype)
            assert np.array_equal(B.retrieve_populations(slot, np.float64), want), (shape, i)


def test_batch_autotune_and_moments():
    sp = specs()
    with lbm.Batch("f32") as B:
        slots = [B.add(*s[:4], s[4], s[5], s[6]) for s in sp]
        info = B.autotune()
        assert info["cells_per_thread"] in (2, 4) and info["block_threads"] % 32 == 0
        B.step(30)
        rho, ux, uy = B.moments(slots[0])
        assert rho.shape == (sp[0][1], sp[0][0])
        assert ux[sp[0][1] - 2, sp[0][0] // 2] > 0  # the lid drags the fluid


def test_moments_tickets_equal_moments_and_survive_removal():
    """lbm_batch_moments_async queues the read-back: its ticket yields the same arrays as the
    waiting read-back even when the slot is removed and others keep stepping before it is
    collected, and collecting without waiting eventually returns the result."""
    sp = specs()
    with lbm.Batch("f16s") as B:
        slots = [B.add(*s[:4], s[4], s[5], s[6]) for s in sp]
        B.set_slot_steps(slots[1], 9)
        B.step(25)
        want = [B.moments(sl) for sl in slots[:3]]
        tickets = [B.moments_async(sl) for sl in slots[:3]]
        B.remove(slots[0])
        B.step(40)  # the others advance; slot 1 has used its budget and stays put
        first = B.collect(tickets[0], wait=False)
        got = [B.collect(t) for t in tickets[1:]]
        while first is None:
            first = B.collect(tickets[0], wait=False)
        got.insert(0, first)
        for w, g in zip(want, got):
            for a, b in zip(w, g):
                assert np.array_equal(a, b)
        assert np.array_equal(B.moments(slots[1])[1], want[1][1])  # slot 1 stopped at its budget
        with pytest.raises(lbm.LBMError):
            B.collect(tickets[1])  # a ticket is collected once
        assert B.info()["slots"] == len(sp) - 1


def test_batch_rejects_bad_input():
    with lbm.Batch("f32") as B:
        with pytest.raises(lbm.LBMError):
            B.add(16, 16, 0.5)
        bad = np.full((8, 8), 5, np.uint8)
        with pytest.raises(lbm.LBMError):
            B.add(8, 8, 0.7, bad)
        with pytest.raises(lbm.LBMError):
            B.remove(3)
        with pytest.raises(lbm.LBMError):
            B.set_launch(8, 32, 1)  # FP32 vectors are 2 or 4 wide


@pytest.mark.parametrize("dtype", ["f32", "f16s"])
def test_many_slots_table_path_and_back(dtype):
    """Past 540 live slots the batch reads its descriptors and tiles from global-memory tables, below
    that from the kernel's parameter block: 600 small slots of varied shape and kind (table path),
    then 120 of them removed mid-run (parameter path), every slot equal to its solo run bit for bit."""
    rng = np.random.default_rng(11)
    kinds = []
    for i in range(600):
        nx, ny = int(rng.integers(3, 70)), int(rng.integers(2, 12))
        per = int(rng.integers(0, 4))
        fl = np.zeros((ny, nx), np.uint8)
        if not per & 2:
            fl[0, :] = 1
            fl[-1, :] = 2 if i % 3 == 0 else 1
        kinds.append((nx, ny, float(rng.uniform(0.55, 1.1)), fl, per, (float(rng.uniform(0, 2e-5)), 0.0),
                      (0.03 if i % 3 == 0 else 0.0, 0.0)))
    first, second = 7, 5
    with lbm.Batch(dtype) as B:
        slots = [B.add(*k[:4], k[4], k[5], k[6]) for k in kinds]
        for i, sl in enumerate(slots):
            B.load_populations(sl, init_state(kinds[i][0], kinds[i][1], 1000 + i))
        B.step(first)
        removed = set(range(0, 600, 5))
        early = {i: B.retrieve_populations(slots[i], np.float64) for i in removed}
        for i in removed:
            B.remove(slots[i])
        B.step(second)
        late = {i: B.retrieve_populations(slots[i], np.float64) for i in range(600) if i not in removed}
    for i, got in early.items():
        assert np.array_equal(got, single(kinds[i], init_state(kinds[i][0], kinds[i][1], 1000 + i), first, dtype)), i
    for i, got in list(late.items())[::7]:
        assert np.array_equal(got, single(kinds[i], init_state(kinds[i][0], kinds[i][1], 1000 + i), first + second,
                                          dtype)), i


@pytest.mark.parametrize("dtype", ["f32", "f16s", "bf16s"])
def test_persistent_launch_equals_one_launch_per_step(dtype):
    """A step sequence run as one persistent (cooperative) launch, its blocks meeting after each
    step, gives the populations of one launch per step, bit for bit, with step budgets that stop
    slots inside the sequence."""
    sp = specs()
    budgets = [5, -1, 9, 0, -1, 3]
    out = {}
    for mode in (0, 2):
        with lbm.Batch(dtype) as B:
            B.set_persistent(mode)
            slots = []
            for i, s in enumerate(sp):
                slot = B.add(*s[:4], s[4], s[5], s[6])
                B.load_populations(slot, init_state(s[0], s[1], 60 + i))
                B.set_slot_steps(slot, budgets[i])
                slots.append(slot)
            B.step(7)
            B.step(6)
            B.synchronize()
            out[mode] = [(B.steps_done(sl), B.retrieve_populations(sl, np.float64)) for sl in slots]
    for i, ((n0, g0), (n2, g2)) in enumerate(zip(out[0], out[2])):
        assert n0 == n2 == (13 if budgets[i] < 0 else min(13, budgets[i]))
        assert np.array_equal(g0, g2), (dtype, i)


def test_persistent_launch_wait_gives_up_and_reports():
    """The persistent launch's bounded meeting, exercised without any fault: with a 1 ms limit and
    block 0 kept from arriving, the other blocks' wait runs out, every block ends the launch, and the
    next lbm_batch_synchronize returns LBM_ERR_TIMEOUT; a new batch afterwards steps as usual."""
    sp = specs()
    with lbm.Batch("f16s") as B:
        B.set_persistent(2, wait_ns=1_000_000, skip_block=0)
        for i, s in enumerate(sp):
            slot = B.add(*s[:4], s[4], s[5], s[6])
            B.load_populations(slot, init_state(s[0], s[1], i))
        B.step(3)
        with pytest.raises(lbm.LBMError) as err:
            B.synchronize()
        assert err.value.status == lbm.capi.ERR_TIMEOUT and "persistent launch" in str(err.value)
        B.synchronize()  # the status was taken: nothing left to report
    s = sp[0]
    with lbm.Batch("f16s") as B:
        slot = B.add(*s[:4], s[4], s[5], s[6])
        B.load_populations(slot, init_state(s[0], s[1], 0))
        B.step(11)
        got = B.retrieve_populations(slot, np.float64)
    assert np.array_equal(got, single(s, init_state(s[0], s[1], 0), 11, "f16s"))
