"""Pin the D2Q9 half of the CPU oracle.  The reference has no D2Q9 code, so the pins are analytic:
conservation, Taylor-Green decay, the Poiseuille profile and Galilean symmetry."""
import numpy as np
import pytest

import oracle


def box_flags(nx, ny, lid=False):
    fl = np.zeros((ny, nx), np.uint8)
    fl[0, :] = 1
    fl[:, 0] = 1
    fl[:, -1] = 1
    fl[-1, :] = 2 if lid else 1
    return fl


def perturbed(nx, ny, seed, amp=1e-2, dtype=np.float64):
    rng = np.random.default_rng(seed)
    rho = 1 + amp * rng.standard_normal((ny, nx))
    ux = amp * rng.standard_normal((ny, nx))
    uy = amp * rng.standard_normal((ny, nx))
    return oracle.d2q9_equilibrium(rho, ux, uy, dtype)


def test_equilibrium_moments():
    f = perturbed(8, 6, 0)
    fl = np.zeros((6, 8), np.uint8)
    rho, ux, uy = oracle.d2q9_moments(f, fl, periodic=3)
    # moments of the streamed populations: total mass is unchanged by streaming
    assert np.isclose(rho.sum(), f.sum(), rtol=1e-13)


@pytest.mark.parametrize("periodic", [0, 1, 3])
def test_mass_conserved_closed(periodic):
    nx, ny = 24, 20
    fl = box_flags(nx, ny) if periodic == 0 else np.zeros((ny, nx), np.uint8)
    if periodic == 1:
        fl[0, :] = 1
        fl[-1, :] = 1
    f0 = perturbed(nx, ny, 1)
    m0 = oracle.d2q9_conservation(f0, fl)
    f = oracle.d2q9_run(f0, fl, 0.7, 300, periodic=periodic)
    m1 = oracle.d2q9_conservation(f, fl)
    assert abs(m1[0] - m0[0]) <= 1e-12 * m0[0]
    if periodic == 3:
        assert np.allclose(m1[1:], m0[1:], atol=1e-12)


def test_force_adds_momentum():
    """Guo forcing on a fully periodic box adds exactly F per fluid cell per step."""
    nx, ny, F = 16, 12, 1e-5
    fl = np.zeros((ny, nx), np.uint8)
    f0 = perturbed(nx, ny, 2)
    m0 = oracle.d2q9_conservation(f0, fl)
    f = oracle.d2q9_run(f0, fl, 0.9, 50, periodic=3, force=(F, -2 * F))
    m1 = oracle.d2q9_conservation(f, fl)
    assert np.isclose(m1[1] - m0[1], 50 * F * nx * ny, rtol=1e-9)
    assert np.isclose(m1[2] - m0[2], -100 * F * nx * ny, rtol=1e-9)


def taylor_green(n, u0, k=None):
    k = 2 * np.pi / n if k is None else k
    x = np.arange(n) + 0.0
    X, Y = np.meshgrid(x, x)
    ux = -u0 * np.cos(k * X) * np.sin(k * Y)
    uy = u0 * np.sin(k * X) * np.cos(k * Y)
    rho = 1 - 0.75 * u0 * u0 * (np.cos(2 * k * X) + np.cos(2 * k * Y))
    return rho, ux, uy


def tgv_decay_error(n, steps, tau, u0=0.02):
    rho, ux, uy = taylor_green(n, u0)
    f = oracle.d2q9_equilibrium(rho, ux, uy)
    fl = np.zeros((n, n), np.uint8)
    f = oracle.d2q9_run(f, fl, tau, steps, periodic=3)
    _, vx, vy = oracle.d2q9_moments(f, fl, periodic=3)
    nu = (tau - 0.5) / 3
    k = 2 * np.pi / n
    amp = (np.sum(vx * ux) + np.sum(vy * uy)) / (np.sum(ux * ux) + np.sum(uy * uy))
    # the moments are those of the streamed populations: time steps + 1
    return amp / np.exp(-2 * nu * k * k * (steps + 1)) - 1


@pytest.mark.parametrize("tau", [0.6, 1.0])
def test_taylor_green_decay(tau):
    """Amplitude follows exp(-2 nu k^2 t), nu = (tau - 1/2)/3, with second-order convergence
    under diffusive scaling (n doubled, steps x4)."""
    e32 = tgv_decay_error(32, 100, tau)
    e64 = tgv_decay_error(64, 400, tau)
    assert abs(e64) < 2e-3
    assert abs(e64) < 0.3 * abs(e32)


def test_poiseuille_profile():
    nx, ny, F, tau = 4, 34, 1e-6, 0.8
    fl = np.zeros((ny, nx), np.uint8)
    fl[0, :] = 1
    fl[-1, :] = 1
    f = oracle.d2q9_equilibrium(np.ones((ny, nx)), np.zeros((ny, nx)), np.zeros((ny, nx)))
    f = oracle.d2q9_run(f, fl, tau, 40000, periodic=1, force=(F, 0.0))
    _, ux, uy = oracle.d2q9_moments(f, fl, periodic=1, force=(F, 0.0))
    nu = (tau - 0.5) / 3
    y = np.arange(1, ny - 1)
    # half-way bounce-back puts the walls half a cell outside the first/last fluid row
    exact = F / (2 * nu) * (y - 0.5) * (ny - 1.5 - y)
    prof = ux[1:-1, 1]
    assert np.max(np.abs(prof - exact)) / exact.max() < 5e-3
    assert np.max(np.abs(uy[1:-1])) < 1e-12


def test_mirror_symmetry():
    """Left/right mirror of a closed box with a mirrored initial state stays mirrored."""
    nx, ny = 20, 16
    fl = box_flags(nx, ny)
    rng = np.random.default_rng(3)
    rho = 1 + 0.01 * rng.standard_normal((ny, nx))
    ux = 0.01 * rng.standard_normal((ny, nx))
    uy = 0.01 * rng.standard_normal((ny, nx))
    rho = 0.5 * (rho + rho[:, ::-1])
    uy = 0.5 * (uy + uy[:, ::-1])
    ux = 0.5 * (ux - ux[:, ::-1])
    f = oracle.d2q9_run(oracle.d2q9_equilibrium(rho, ux, uy), fl, 0.65, 100)
    r, vx, vy = oracle.d2q9_moments(f, fl)
    assert np.allclose(r, r[:, ::-1], atol=1e-13)
    assert np.allclose(vx, -vx[:, ::-1], atol=1e-13)
    assert np.allclose(vy, vy[:, ::-1], atol=1e-13)


def test_lid_drives_cavity():
    nx = ny = 32
    fl = box_flags(nx, ny, lid=True)
    f = oracle.d2q9_equilibrium(np.ones((ny, nx)), np.zeros((ny, nx)), np.zeros((ny, nx)))
    f = oracle.d2q9_run(f, fl, 0.6, 500, wall_velocity=(0.05, 0.0))
    _, ux, _ = oracle.d2q9_moments(f, fl, wall_velocity=(0.05, 0.0))
    assert ux[ny - 2, nx // 2] > 0.01
    assert ux[ny // 3, nx // 2] < 0


def test_f32_tracks_f64():
    nx = ny = 48
    fl = box_flags(nx, ny, lid=True)
    f64 = oracle.d2q9_equilibrium(np.ones((ny, nx)), np.zeros((ny, nx)), np.zeros((ny, nx)))
    a = oracle.d2q9_run(f64, fl, 0.6, 300, wall_velocity=(0.05, 0.0))
    b = oracle.d2q9_run(f64.astype(np.float32), fl, np.float32(0.6), 300, wall_velocity=(0.05, 0.0))
    assert np.max(np.abs(a - b)) < 1e-5


def test_oracle_channel_flags_equal_the_library_generator():
    """The CPU baseline builds the benchmark channel with the oracle's restatement of the seeded
    generator; it must give the library's bytes (the headline channel and smaller cases)."""
    import latticeboltzmanncuda_gb300 as lbm
    for args in ((4096, 1024, 64, 8.0, 24.0, 20261203), (300, 77, 9, 3.0, 9.5, 1), (64, 20, 2, 2.0, 4.0, 3)):
        want, _ = lbm.gen_channel(*args)
        assert np.array_equal(oracle.channel_flags(*args), want), args
