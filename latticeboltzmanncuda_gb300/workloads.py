"""Seeded synthetic workloads: lid-driven cavity, obstacle channel, Taylor-Green vortex, batches of
uneven domains and a Poisson stream of solve requests.  Flag masks come from the library's
SplitMix64 generators; the sampled sizes and parameters use numpy's PCG64 seeded with the same
seed, so every workload is a pure function of its seed."""
from __future__ import annotations

import math
from dataclasses import dataclass

import numpy as np

from . import gen_cavity, gen_channel, gen_disks_fraction

DEFAULT_SEED = 20261203


@dataclass
class Domain:
    nx: int
    ny: int
    tau: float
    flags: np.ndarray
    periodic: int = 0
    body_force: tuple = (0.0, 0.0)
    wall_velocity: tuple = (0.0, 0.0)
    drive: str = "lid"
    solid_fraction: float = 0.0
    steps: int = 0
    arrival: float = 0.0  # seconds after the start of a request stream
    rid: int = 0

    @property
    def cells(self):
        return self.nx * self.ny


def cavity(n=128, lid=0.05, tau=0.6):
    return Domain(n, n, tau, gen_cavity(n, n), 0, (0.0, 0.0), (lid, 0.0), "lid")


def channel(nx=4096, ny=1024, ndisks=64, rmin=8.0, rmax=24.0, force=1e-6, tau=0.55, seed=DEFAULT_SEED):
    flags, _ = gen_channel(nx, ny, ndisks, rmin, rmax, seed)
    return Domain(nx, ny, tau, flags, 1, (force, 0.0), (0.0, 0.0), "force")


def taylor_green_fields(n, u0=0.04):
    """Initial density and velocity of the periodic Taylor-Green vortex, k = 2 pi / n."""
    k = 2 * math.pi / n
    x = np.arange(n, dtype=np.float64)
    X, Y = np.meshgrid(x, x)
    ux = -u0 * np.cos(k * X) * np.sin(k * Y)
    uy = u0 * np.sin(k * X) * np.cos(k * Y)
    rho = 1 - 0.75 * u0 * u0 * (np.cos(2 * k * X) + np.cos(2 * k * Y))
    return rho, ux, uy


def _random_domain(rng, seed, area_lo, area_hi, aspect_hi, tau_lo, tau_hi, solid_hi):
    a, b = float(area_lo), float(area_hi)
    area = math.exp(rng.uniform(math.log(a), math.log(b)))
    aspect = rng.uniform(1.0, aspect_hi)
    nx = max(8, int(round(math.sqrt(area * aspect))))
    ny = max(8, int(round(math.sqrt(area / aspect))))
    if rng.uniform() < 0.5:
        nx, ny = ny, nx
    tau = float(rng.uniform(tau_lo, tau_hi))
    solid = float(rng.uniform(0.0, solid_hi))
    lid = rng.uniform() < 0.5
    if lid:
        flags = gen_cavity(nx, ny)
        per, force, wall, drive = 0, (0.0, 0.0), (0.05, 0.0), "lid"
    else:
        flags = np.zeros((ny, nx), np.uint8)
        flags[0, :] = 1
        flags[-1, :] = 1
        per, force, wall, drive = 1, (1e-6, 0.0), (0.0, 0.0), "force"
    side = min(nx, ny)
    flags, achieved = gen_disks_fraction(flags, solid, max(1.0, side / 32), max(2.0, side / 10), seed)
    return Domain(nx, ny, tau, flags, per, force, wall, drive, achieved)


def batch(count=512, seed=DEFAULT_SEED, steps=2000):
    """Independent domains: area log-uniform in [64^2, 1024^2], aspect ratio uniform in [1, 4] with
    random orientation, tau uniform in [0.52, 1.2], random disks up to a solid fraction uniform in
    [0, 0.3], lid-driven (lid 0.05) or body-forced (1e-6, periodic x) with probability 1/2."""
    rng = np.random.default_rng(seed)
    out = []
    for i in range(count):
        d = _random_domain(rng, seed * 1000003 + i, 64 * 64, 1024 * 1024, 4.0, 0.52, 1.2, 0.30)
        d.steps = steps
        out.append(d)
    return out


def small_batch(count, seed=DEFAULT_SEED):
    """`count` small independent domains (area log-uniform in [64^2, 256^2], otherwise as batch()):
    a batch whose step is short enough for the launch of each step to matter."""
    rng = np.random.default_rng(seed + 11)
    return [_random_domain(rng, seed * 31 + i, 64 * 64, 256 * 256, 4.0, 0.52, 1.2, 0.30) for i in range(count)]


def requests(rate, duration, seed=DEFAULT_SEED, side_lo=128, side_hi=2048, steps_lo=1000, steps_hi=50000):
    """Poisson arrivals at `rate` per second for `duration` seconds.  Side length log-uniform in
    [side_lo, side_hi] (area = side^2, aspect as in batch()), solid 0-30 %, tau 0.52-1.2, steps
    log-uniform in [steps_lo, steps_hi].  Returns Domains with `arrival` and `rid` set."""
    rng = np.random.default_rng(seed + 7)
    t, out, i = 0.0, [], 0
    while True:
        t += rng.exponential(1.0 / rate)
        if t > duration:
            break
        side = math.exp(rng.uniform(math.log(side_lo), math.log(side_hi)))
        d = _random_domain(rng, seed * 7919 + i, side * side, side * side * 1.0000001, 4.0, 0.52, 1.2, 0.30)
        d.steps = int(round(math.exp(rng.uniform(math.log(steps_lo), math.log(steps_hi)))))
        d.arrival, d.rid = t, i
        out.append(d)
        i += 1
    return out
