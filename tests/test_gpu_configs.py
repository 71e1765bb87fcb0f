"""Parity at the benchmark configurations' own sizes (D2Q9; the reference has no D2Q9, so the
FP64 GPU run is the oracle here -- it is itself pinned to the CPU FP64 oracle to 1e-12 by
test_gpu_d2q9.py::test_fp64_gpu_matches_fp64_oracle on every boundary kind these runs use).

Error measures (u = (ux, uy) per cell, all cells that are not solid):
  velocity  L2   sqrt(sum |u - u64|^2 / sum |u64|^2)       max   max |u - u64| / max |u64|
  density   L2   sqrt(sum (rho - rho64)^2 / sum (rho64 - 1)^2), rho = the sum of a cell's stored
            populations read back in FP64 (relative to the density deviation, the part of rho that
            carries information: relative to rho itself it would be ~1e-7, and the FP32 density of
            lbm_moments is itself quantised to 6e-8, of the order of the deviation in the channel)

Tolerances (stated here, asserted below):
  C2 channel 4096 x 1024, 64 disks, 10,000 steps, FP32 storage:
      max |f - f64| <= 1e-5 max |f|;  velocity L2 <= 3e-4, max <= 5e-4;  density L2 <= 1e-2
      (FP32 rounding of the stored populations, repeated in nearly the same way step after step in a
      slowly changing flow, accumulates to ~1e-4 of the velocity over 10,000 steps)
  C3 Taylor-Green 2048^2, 5000 steps, tau in {0.51, 0.6, 1.0}:
      FP32   velocity L2 vs FP64 <= 3e-4, density L2 <= 2e-3
      FP16s  velocity L2 vs FP64 <= 1e-3 (the benchmark target), density L2 <= 3e-2
      BF16s  velocity L2 vs FP64 <= 2e-2, density L2 <= 0.3 (8-bit significand: stated, not a target)
      against the analytic decay u0 exp(-2 nu k^2 t): FP64, FP32, FP16s within 2e-3, BF16s within 2e-2
  C4 mix (32 of the 512 seeded batch domains, 2000 steps, batched):
      FP16s  velocity L2 vs FP64 <= 1e-3 on every domain (the benchmark target);  FP32 <= 1e-4
Each test prints one PARITY line with the measured figures (pytest -s).
"""
import json
import math

import numpy as np
import pytest

import latticeboltzmanncuda_gb300 as lbm
from latticeboltzmanncuda_gb300 import workloads

pytestmark = pytest.mark.gpu

SEED = 20261203


def report(name, **figs):
    print("PARITY " + json.dumps({"case": name, **figs}, default=float), flush=True)


def vel_err(u, v, u64, v64, mask):
    du2 = (u - u64) ** 2 + (v - v64) ** 2
    ref2 = u64 ** 2 + v64 ** 2
    l2 = math.sqrt(float(np.sum(du2[mask])) / max(float(np.sum(ref2[mask])), 1e-300))
    mx = math.sqrt(float(np.max(du2[mask]))) / max(math.sqrt(float(np.max(ref2[mask]))), 1e-300)
    return l2, mx


def rho_err(r, r64, mask):
    d = (r.astype(np.float64) - r64)[mask]
    dev = (r64 - 1.0)[mask]
    return math.sqrt(float(np.sum(d * d)) / max(float(np.sum(dev * dev)), 1e-300))


def run_single(nx, ny, dtype, tau, steps, flags=None, periodic=0, force=(0.0, 0.0), wall=(0.0, 0.0), init=None,
               populations=False):
    with lbm.Lattice(nx, ny, dtype=dtype, tau=tau, periodic=periodic, body_force=(*force, 0.0),
                     wall_velocity=(*wall, 0.0)) as L:
        if flags is not None:
            L.set_flags(flags)
        if init is None:
            L.init_equilibrium()
        else:
            L.init_equilibrium(*init)
        L.step(steps)
        _, ux, uy = (a.astype(np.float64) for a in L.moments())
        f = L.retrieve_populations(np.float64)
    rho = f.sum(axis=0)
    return (f if populations else None), rho, ux, uy


def test_c2_channel_full_size_fp32_against_fp64():
    """C2 as benchmarked: 4096 x 1024, periodic x, walls at y = 0 and 1023, Guo force 1e-6, tau 0.55,
    64 seeded non-overlapping disks r in [8, 24], 10,000 steps.  FP32 storage against FP64 storage."""
    nx, ny, steps = 4096, 1024, 10000
    flags, disks = lbm.gen_channel(nx, ny, 64, 8.0, 24.0, SEED)
    assert len(disks) == 64
    kw = dict(flags=flags, periodic=1, force=(1e-6, 0.0), populations=True)
    f64, r64, u64, v64 = run_single(nx, ny, "f64", 0.55, steps, **kw)
    f32, r32, u32, v32 = run_single(nx, ny, "f32", 0.55, steps, **kw)
    fluid = flags == 0
    fmax = float(np.max(np.abs(f64[:, fluid])))
    df = float(np.max(np.abs(f32 - f64)[:, fluid]))
    del f64, f32
    l2, mx = vel_err(u32, v32, u64, v64, fluid)
    rl2 = rho_err(r32, r64, fluid)
    report("C2 channel fp32", max_df_rel=df / fmax, vel_l2=l2, vel_max=mx, rho_l2=rl2,
           umax=float(np.max(np.hypot(u64, v64)[fluid])))
    assert df <= 1e-5 * fmax, (df, fmax)
    assert l2 <= 3e-4 and mx <= 5e-4, (l2, mx)
    assert rl2 <= 1e-2, rl2


@pytest.mark.parametrize("tau", [0.51, 0.6, 1.0])
def test_c3_taylor_green_2048_every_storage_type(tau):
    """C3 as benchmarked: Taylor-Green vortex 2048^2, periodic, u0 0.04, 5000 steps; FP32, FP16- and
    BF16-shifted storage against the FP64 run of the same grid, and every run against the analytic
    decay."""
    n, steps, u0 = 2048, 5000, 0.04
    rho0, ux0, uy0 = workloads.taylor_green_fields(n, u0)
    init = (rho0, ux0, uy0)
    k = 2 * math.pi / n
    nu = (float(np.float32(tau)) - 0.5) / 3
    decay = math.exp(-2 * nu * k * k * (steps + 1))  # moments are those of the streamed populations
    ua, va = ux0 * decay, uy0 * decay
    everywhere = np.ones((n, n), bool)
    _, r64, u64, v64 = run_single(n, n, "f64", tau, steps, periodic=3, init=init)
    figs = {"f64": {"vs_analytic": vel_err(u64, v64, ua, va, everywhere)[0]}}
    bounds = {"f32": (3e-4, 2e-3), "f16s": (1e-3, 3e-2), "bf16s": (2e-2, 0.3)}
    for dtype in ("f32", "f16s", "bf16s"):
        _, r, u, v = run_single(n, n, dtype, tau, steps, periodic=3, init=init)
        l2, mx = vel_err(u, v, u64, v64, everywhere)
        figs[dtype] = {"vel_l2": l2, "vel_max": mx, "rho_l2": rho_err(r, r64, everywhere),
                       "vs_analytic": vel_err(u, v, ua, va, everywhere)[0]}
    report(f"C3 taylor-green tau {tau}", **figs)
    for dtype, (vb, rb) in bounds.items():
        assert figs[dtype]["vel_l2"] <= vb, (dtype, figs[dtype])
        assert figs[dtype]["rho_l2"] <= rb, (dtype, figs[dtype])
    for dtype, f in figs.items():
        assert f["vs_analytic"] <= (2e-2 if dtype == "bf16s" else 2e-3), (dtype, f)


def test_c4_mix_batched_16bit_within_target():
    """C4 domains (the seeded 512-domain batch: uneven sizes, tau 0.52-1.2, 0-30 % solid, lid-driven
    or body-forced), 32 of them advanced together for 2000 steps in FP16-shifted and FP32 storage,
    each against its own FP64 run (the batched FP64 path equals the single-domain FP64 path bit for
    bit, test_gpu_batch.py)."""
    doms = workloads.batch(512, SEED, 2000)
    pick = [doms[i] for i in range(0, 512, 16)]
    out = {}
    for dtype in ("f64", "f32", "f16s"):
        with lbm.Batch(dtype) as B:
            slots = [B.add(d.nx, d.ny, d.tau, d.flags, d.periodic, d.body_force, d.wall_velocity) for d in pick]
            B.step(2000)
            out[dtype] = [(B.retrieve_populations(s, np.float64).sum(axis=0),
                           *(a.astype(np.float64) for a in B.moments(s)[1:])) for s in slots]
    errs = {"f32": [], "f16s": []}
    for i, d in enumerate(pick):
        fluid = d.flags == 0
        r64, u64, v64 = out["f64"][i]
        for dtype in errs:
            r, u, v = out[dtype][i]
            l2, mx = vel_err(u, v, u64, v64, fluid)
            errs[dtype].append((l2, mx, rho_err(r, r64, fluid)))
    summary = {dt: {"vel_l2_max": max(e[0] for e in v), "vel_l2_median": float(np.median([e[0] for e in v])),
                    "vel_max_max": max(e[1] for e in v), "rho_l2_max": max(e[2] for e in v)}
               for dt, v in errs.items()}
    worst = int(np.argmax([e[0] for e in errs["f16s"]]))
    d = pick[worst]
    summary["f16s_worst_domain"] = {"nx": d.nx, "ny": d.ny, "tau": d.tau, "drive": d.drive,
                                    "solid": d.solid_fraction}
    report("C4 mix batched", domains=len(pick), **summary)
    assert summary["f16s"]["vel_l2_max"] <= 1e-3, summary
    assert summary["f32"]["vel_l2_max"] <= 1e-4, summary
