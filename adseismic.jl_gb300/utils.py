"""Input generation helpers mirroring src/Utils.jl (wavelets, material transforms)
and the seeded synthetic models the benchmarks and tests run on."""
from __future__ import annotations

import math

import numpy as np


def Ricker(param, a, shift, amp=1.0):
    """src/Utils.jl:188-204: amp*A*(1 - x^2/a^2)*exp(-x^2/(2a^2)), x = 1..NSTEP - shift,
    A = 2/(sqrt(3a) pi^(1/4)); `a` and `shift` are in samples."""
    NT = int(param.NSTEP)
    A = 2 / (math.sqrt(3 * a) * (math.pi ** 0.25))
    wsq = a * a
    vec = np.arange(1, NT + 1, dtype=np.float64) - shift
    xsq = vec * vec
    return amp * A * (1 - xsq / wsq) * np.exp(-xsq / (2 * wsq))


def ricker_width_samples(fpeak, dt):
    """Ricker width `a` (in samples) for a peak frequency: a = 1/(pi f sqrt(2) dt)."""
    return 1.0 / (math.pi * fpeak * math.sqrt(2.0) * dt)


def Gauss(param, a, shift=None, amp=1.0):
    """src/Utils.jl:206-220: amp*2*A*exp(-A (t - shift)^2), A = pi^2 a^2, t = (0..NSTEP-1) dt."""
    if shift is None:
        shift = 1.2 / a
    t = np.arange(param.NSTEP, dtype=np.float64) * param.DELTAT
    A = math.pi ** 2 * a ** 2
    return amp * 2.0 * A * np.exp(-A * (t - shift) ** 2)


def compute_lame_parameters(vp, vs, rho):
    """src/Utils.jl:237-243: mu = rho vs vs, lambda = rho (vp vp - 2 vs vs)."""
    vp, vs, rho = (np.asarray(x, dtype=np.float64) for x in (vp, vs, rho))
    mu = rho * vs * vs
    lam = rho * (vp * vp - 2.0 * vs * vs)
    return lam, mu, rho


def compute_properties(vp, vs, rho):
    """src/Utils.jl:249-258: mu = rho vs vs, lambda = rho vp vp - 2 mu."""
    vp, vs, rho = (np.asarray(x, dtype=np.float64) for x in (vp, vs, rho))
    mu = rho * vs * vs
    lam = rho * vp * vp - 2 * mu
    return lam, mu, rho


# ------------------------------------------------------------------ synthetic models

def layered_gaussian_model(nx2, ny2, vmin=2000.0, vmax=3500.0, sigma=15.0, amp=0.10,
                           seed=0):
    """Layered vmin->vmax with a linear depth gradient plus a seeded Gaussian
    anomaly (+-amp, width sigma cells).  Shape (nx2, ny2), depth = axis 1."""
    rng = np.random.default_rng(seed)
    j = np.arange(ny2, dtype=np.float64)
    nlay = 4
    edges = np.linspace(0, ny2, nlay + 1)
    base = np.empty(ny2)
    for k in range(nlay):
        m = (j >= edges[k]) & (j < edges[k + 1])
        base[m] = vmin + (vmax - vmin) * k / (nlay - 1) * 0.8
    base += (vmax - vmin) * 0.2 * j / max(ny2 - 1, 1)
    vp = np.repeat(base[None, :], nx2, axis=0)
    ci, cj = nx2 / 2 + rng.uniform(-0.1, 0.1) * nx2, ny2 / 2 + rng.uniform(-0.1, 0.1) * ny2
    sign = 1.0 if rng.random() < 0.5 else -1.0
    ii, jj = np.meshgrid(np.arange(nx2), j, indexing="ij")
    vp *= 1 + sign * amp * np.exp(-((ii - ci) ** 2 + (jj - cj) ** 2) / (2 * sigma ** 2))
    return vp


def folded_layer_model(nx2, ny2, vmin=1500.0, vmax=4500.0, seed=0):
    """3-6 folded interfaces z_k(x) = z0_k + A_k sin(2 pi x / L_k + phi_k), layer
    velocities drawn in [vmin, vmax] increasing with depth (seeded)."""
    rng = np.random.default_rng(seed)
    n = int(rng.integers(3, 7))
    z0 = np.sort(rng.uniform(0.1, 0.9, n)) * ny2
    A = rng.uniform(0.02, 0.08, n) * ny2
    L = rng.uniform(0.3, 1.5, n) * nx2
    ph = rng.uniform(0, 2 * np.pi, n)
    vel = np.sort(rng.uniform(vmin, vmax, n + 1))
    x = np.arange(nx2, dtype=np.float64)[:, None]
    z = np.arange(ny2, dtype=np.float64)[None, :]
    vp = np.full((nx2, ny2), vel[0])
    for k in range(n):
        zk = z0[k] + A[k] * np.sin(2 * np.pi * x / L[k] + ph[k])
        vp = np.where(z >= zk, vel[k + 1], vp)
    return vp


def gaussian_smooth(v, sigma):
    """Separable Gaussian blur with edge padding (start models)."""
    from scipy.ndimage import gaussian_filter

    return gaussian_filter(np.asarray(v, dtype=np.float64), sigma=sigma, mode="nearest")
