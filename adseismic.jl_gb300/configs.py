"""Seeded synthetic workloads of the five benchmark configurations.

The benchmark and the tests build their inputs here, so a test at a
configuration's full size runs on exactly what the benchmark times.  Every
model, wavelet and geometry is drawn from a fixed seed (numpy default_rng).

  C1  acoustic forward, plain FP64: 200 x 200 interior + PML 20 (NX = NY = 240),
      h = 10 m, dt = 1 ms, 1000 steps, one 10 Hz Ricker source 20 cells below
      the PML, 200 receivers 5 cells below it.
  C2  acoustic FWI gradient, plain FP64: 400 x 400 including PML 30, 2000 steps,
      8 shots at the centres of 8 equal interior segments, one receiver per
      interior column; observed data from the true model, gradient at a
      start model smoothed by 5% of the grid width (20 cells).
  C3  batched acoustic FWI gradient, FP32 stencils: 1000 x 500 (PML 40),
      h = 10 m, dt = 0.8 ms, 3000 steps, 64 shots with 15 Hz Ricker wavelets
      and 500 receivers each, folded-layer model 1500-4500 m/s.
  C4  elastic CPML gradient w.r.t. lambda, mu, rho: 600 x 300 (CPML 30),
      h = 10 m, dt = 0.8 ms, 4000 steps, 32 explosive shots (sigma_xx and
      sigma_yy, 10 Hz Ricker), 300 two-component receivers; vp layered
      2500-5000 m/s, vs = vp / sqrt(3) with +-5% noise, rho = 310 vp^0.25.
  C5  uneven batched acoustic gradient on a 4000 x 2000 layered-plus-anomaly
      model: 128 shots with windows 400-1200 columns (PML 40 inside each),
      200-1200 receivers and 2000-6000 steps, all drawn from the seed.

Shot dictionaries are the ones AcousticPlan / ElasticPlan take.
"""
from __future__ import annotations

import numpy as np

from .acoustic import AcousticPropagatorParams
from .elastic import ElasticPropagatorParams
from .utils import (Ricker, compute_properties, folded_layer_model, gaussian_smooth,
                    layered_gaussian_model, ricker_width_samples)


def _ricker(nstep, dt, fpeak):
    p = AcousticPropagatorParams(NSTEP=nstep, DELTAT=dt)
    return Ricker(p, ricker_width_samples(fpeak, dt), 1.5 / fpeak / dt, 1e6)


def c1_forward():
    """C1: (cfg, shot, vp)."""
    NX = NY = 240
    npml, T, h, dt = 20, 1000, 10.0, 1e-3
    vp = layered_gaussian_model(NX + 2, NY + 2, 2000.0, 3500.0, seed=7)
    wav = _ricker(T, dt, 10.0)
    shot = dict(x0=0, nx=NX, nstep=T, srci=[NX // 2 + 1], srcj=[npml + 21], srcv=wav[:, None],
                rcvi=np.arange(npml + 2, npml + 202), rcvj=np.full(200, npml + 6))
    cfg = dict(MX=NX, MY=NY, h=h, dt=dt, npml=npml, vp_ref=float(vp.mean()), nstep=T)
    return cfg, shot, vp


def c2_fwi(nstep=2000):
    """C2: (cfg, shots, vp_true, vp_start)."""
    NX = NY = 400
    npml, h, dt = 30, 10.0, 1e-3
    vt = layered_gaussian_model(NX + 2, NY + 2, 2000.0, 3500.0, seed=11)
    v0 = gaussian_smooth(vt, 0.05 * NX)
    wav = _ricker(nstep, dt, 10.0)
    seg = (NX - 2 * npml) / 8
    shots = [dict(x0=0, nx=NX, nstep=nstep, srci=[int(npml + 1 + (k + 0.5) * seg) + 1],
                  srcj=[npml + 21], srcv=wav[:, None],
                  rcvi=np.arange(npml + 2, NX - npml + 2), rcvj=np.full(NX - 2 * npml, npml + 6))
             for k in range(8)]
    cfg = dict(MX=NX, MY=NY, h=h, dt=dt, npml=npml, vp_ref=float(vt.mean()), nstep=nstep)
    return cfg, shots, vt, v0


def c3_batched(nshots=64, nstep=3000, seed=1234, MX=1000, MY=500, npml=40, nrcv=500,
               fpeak=15.0, dt=0.8e-3, h=10.0):
    """C3: (cfg, shots, vp_true, vp_start).  Shots sit 11 cells below the PML,
    evenly along x; receivers 6 cells below it, evenly over the interior."""
    vp_true = folded_layer_model(MX + 2, MY + 2, 1500.0, 4500.0, seed=seed)
    vp0 = gaussian_smooth(vp_true, sigma=0.05 * MX)
    wav = _ricker(nstep, dt, fpeak)
    lo, hi = npml + 2, MX - npml
    rcvi = np.round(np.linspace(npml + 2, MX - npml, nrcv)).astype(np.int64)
    shots = []
    for s in range(nshots):
        si = int(round(lo + (s + 0.5) * (hi - lo) / nshots))
        shots.append(dict(x0=0, nx=MX, nstep=nstep, srci=[si], srcj=[npml + 11],
                          srcv=wav[:, None], rcvi=rcvi, rcvj=np.full(nrcv, npml + 6)))
    cfg = dict(MX=MX, MY=MY, h=h, dt=dt, npml=npml, vp_ref=float(vp_true.mean()),
               nstep=nstep)
    return cfg, shots, vp_true, vp0


def c4_elastic(nshots=32, NX=600, NY=300, npml=30, T=4000, h=10.0, dt=0.8e-3, fpeak=10.0,
               seed=5):
    """C4: (param, shots, lambda, mu, rho), the true model on the (NX+2, NY+2) grid."""
    rng = np.random.default_rng(seed)
    j = np.arange(NY + 2, dtype=np.float64)
    vp1 = 2500.0 + 2500.0 * np.floor(j / (NY + 2) * 5) / 4
    vp = np.repeat(vp1[None, :], NX + 2, axis=0)
    vs = vp / np.sqrt(3) * (1 + 0.05 * (2 * rng.random(vp.shape) - 1))
    rho = 310.0 * vp ** 0.25
    lam, mu, rho = compute_properties(vp, vs, rho)
    p = ElasticPropagatorParams(NX=NX, NY=NY, NSTEP=T, DELTAX=h, DELTAY=h, DELTAT=dt,
                                NPOINTS_PML=npml, vp_ref=float(vp.mean()), f0=fpeak)
    wav = _ricker(T, dt, fpeak)
    xr = np.round(np.linspace(npml + 2, NX - npml, 300)).astype(np.int64)
    shots = []
    for s in range(nshots):
        si = int(round(npml + 2 + (s + 0.5) * (NX - 2 * npml - 2) / nshots))
        shots.append(dict(srci=[si, si], srcj=[npml + 11] * 2, srctype=[2, 3],
                          srcv=np.repeat(wav[:, None], 2, axis=1),
                          rcvi=np.concatenate([xr, xr]), rcvj=np.full(600, npml + 6),
                          rcvtype=np.array([0] * 300 + [1] * 300)))
    return p, shots, lam, mu, rho


def c4_start_model(lam, mu, rho, sigma=10.0):
    """The smoothed start model the C4 gradient is taken at."""
    return tuple(gaussian_smooth(a, sigma) for a in (lam, mu, rho))


def c5_uneven(nshots=128, MX=4000, MY=2000, npml=40, h=10.0, dt=0.8e-3, seed=2025):
    """C5: (cfg, shots, vp_true, vp_start); shots in seed order."""
    rng = np.random.default_rng(seed)
    vt = folded_layer_model(MX + 2, MY + 2, 1500.0, 4500.0, seed=seed)
    ii, jj = np.meshgrid(np.arange(MX + 2), np.arange(MY + 2), indexing="ij")
    for _ in range(6):
        ci, cj = rng.uniform(0, MX), rng.uniform(0.2 * MY, MY)
        vt *= 1 + rng.uniform(-0.1, 0.1) * np.exp(-((ii - ci) ** 2 + (jj - cj) ** 2) /
                                                 (2 * 60.0 ** 2))
    v0 = gaussian_smooth(vt, 40.0)
    shots = []
    for s in range(nshots):
        W = int(rng.integers(400, 1201))
        x0 = int(rng.integers(0, MX - W + 1))
        T = int(rng.integers(2000, 6001))
        R = min(int(rng.integers(200, 1201)), W - 2 * npml)
        wav = _ricker(T, dt, 15.0)
        shots.append(dict(x0=x0, nx=W, nstep=T, srci=[int(rng.integers(npml + 2, W - npml))],
                          srcj=[npml + 11], srcv=wav[:, None],
                          rcvi=np.round(np.linspace(npml + 2, W - npml, R)).astype(np.int64),
                          rcvj=np.full(R, npml + 6)))
    cfg = dict(MX=MX, MY=MY, h=h, dt=dt, npml=npml, vp_ref=float(vt.mean()))
    return cfg, shots, vt, v0


def acoustic_plan(ads, cfg, shots, precision, **kw):
    """An AcousticPlan over `shots` of a workload's model."""
    return ads.AcousticPlan(cfg["MX"], cfg["MY"], cfg["h"], cfg["h"], cfg["dt"], shots,
                            npml=cfg["npml"], vp_ref=cfg["vp_ref"], precision=precision, **kw)


def per_trace_rel(a, b, nrcv, floor=1e-6):
    """rel-L2 of every receiver trace (columns of the (nstep+1, nrcv) records)
    of a against b.  Traces whose reference norm is below `floor` times the
    largest trace norm are skipped: they hold only the scheme's numerical
    precursor (values far below FP32's normal range), not signal."""
    a = np.asarray(a, dtype=np.float64).reshape(-1, nrcv)
    b = np.asarray(b, dtype=np.float64).reshape(-1, nrcv)
    nb = np.linalg.norm(b, axis=0)
    m = nb > floor * nb.max() if nb.size and nb.max() > 0 else nb > 0
    return np.linalg.norm(a - b, axis=0)[m] / nb[m]
