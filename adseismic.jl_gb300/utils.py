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


def compute_lame_parameters(*args):
    """src/Utils.jl:223-243: compute_lame_parameters(vp, vs, rho) on arrays,
    mu = rho vs vs, lambda = rho (vp vp - 2 vs vs); or
    compute_lame_parameters(NX, NY, vp, vs, rho) with scalars, the same
    values filled into (NX+2, NY+2) grids.  Returns (lambda, mu, rho)."""
    if len(args) == 5:
        NX, NY, vp, vs, rho = args
        shape = (int(NX) + 2, int(NY) + 2)
        return (np.full(shape, rho * (vp * vp - 2.0 * vs * vs)), np.full(shape, rho * vs * vs),
                np.full(shape, float(rho)))
    if len(args) != 3:
        raise TypeError("compute_lame_parameters(vp, vs, rho) or (NX, NY, vp, vs, rho)")
    vp, vs, rho = (np.asarray(x, dtype=np.float64) for x in args)
    mu = rho * vs * vs
    lam = rho * (vp * vp - 2.0 * vs * vs)
    return lam, mu, rho


def compute_properties(vp, vs, rho):
    """src/Utils.jl:249-258: mu = rho vs vs, lambda = rho vp vp - 2 mu."""
    vp, vs, rho = (np.asarray(x, dtype=np.float64) for x in (vp, vs, rho))
    mu = rho * vs * vs
    lam = rho * vp * vp - 2 * mu
    return lam, mu, rho


def compute_properties_grad(vp, vs, rho, grad_lambda, grad_mu, grad_rho):
    """Chain rule of compute_properties (src/Utils.jl:249-258: mu = rho vs^2,
    lambda = rho vp^2 - 2 mu, rho passed through): from the gradients of a
    loss with respect to lambda, mu and rho, as the elastic plans return them,
    the gradients with respect to vp, vs and rho, which the reference's
    elastic inversion (inv_vp / inv_vs / inv_rho, src/IO.jl:27-40) trains.
    Elementwise; takes numpy arrays or torch tensors (on any device)."""
    g_vp = 2.0 * rho * vp * grad_lambda
    g_vs = 2.0 * rho * vs * (grad_mu - 2.0 * grad_lambda)
    g_rho = grad_rho + (vp * vp - 2.0 * vs * vs) * grad_lambda + vs * vs * grad_mu
    return g_vp, g_vs, g_rho


def gradtest(fg, x, direction=None, seed=0):
    """Taylor-remainder gradient check of src/Utils.jl:260-289, without the
    plot: with G = grad L(x) and a direction v (default uniform [0, 1) times
    median(x), as the reference draws it), for gamma = 1e-1 .. 1e-5 returns
    (gammas, s, w) where s = L(x + gamma v) - L(x) shrinks as O(gamma) and
    w = s - gamma <v, G> as O(gamma^2) when G is right.  fg(x) -> (loss,
    gradient), numpy vectors (a plan's gradient, flattened, works)."""
    x = np.asarray(x, dtype=np.float64)
    L, G = fg(x)
    G = np.asarray(G, dtype=np.float64).reshape(x.shape)
    if direction is None:
        direction = np.random.default_rng(seed).random(x.shape) * np.median(x)
    v = np.asarray(direction, dtype=np.float64).reshape(x.shape)
    gammas = 1.0 / 10.0 ** np.arange(1, 6)
    s = np.empty(5)
    w = np.empty(5)
    for k, g in enumerate(gammas):
        Li = float(fg(x + g * v)[0])
        s[k] = Li - float(L)
        w[k] = s[k] - g * float(np.sum(v * G))
    return gammas, s, w


def add_initial_model(x, v):
    """src/Utils.jl:140-166: add x (a model update, or a stack of them along
    the first axis) to the model v, centred: x smaller than v is added into
    v's centre, x larger than v contributes its centred window of v's size."""
    x = np.asarray(x, dtype=np.float64)
    v = np.asarray(v, dtype=np.float64)
    sx = x.shape[1:] if x.ndim == 3 else x.shape
    if sx[0] <= v.shape[0] and sx[1] <= v.shape[1]:
        i0, j0 = (v.shape[0] - sx[0]) // 2, (v.shape[1] - sx[1]) // 2
        out = np.repeat(v[None], x.shape[0], axis=0) if x.ndim == 3 else v.copy()
        out[..., i0:i0 + sx[0], j0:j0 + sx[1]] += x
        return out
    if sx[0] >= v.shape[0] and sx[1] >= v.shape[1]:
        i0, j0 = (sx[0] - v.shape[0]) // 2, (sx[1] - v.shape[1]) // 2
        return v + x[..., i0:i0 + v.shape[0], j0:j0 + v.shape[1]]
    raise ValueError(f"size error: model {v.shape}, update {sx}")


# ------------------------------------------------------------------ variable sources

def _source_cells(param, srctype):
    """1-based (i, j) of the padded-grid cells a plan accepts as source cells,
    in the reference's row-major order (j fastest): the interior
    2..NX+1 x 2..NY+1 for acoustic parameters; for elastic ones the cells the
    stencil of field `srctype` updates (vx 3..NX+1 x 3..NY+1, vy 2..NX x 2..NY,
    sxx / syy 2..NX x 3..NY+1, sxy 3..NX+1 x 2..NY; src/Core.jl:96-213)."""
    NX, NY = int(param.NX), int(param.NY)
    if srctype is None:
        ri, rj = (2, NX + 1), (2, NY + 1)
    else:
        boxes = {0: ((3, NX + 1), (3, NY + 1)), 1: ((2, NX), (2, NY)),
                 2: ((2, NX), (3, NY + 1)), 3: ((2, NX), (3, NY + 1)),
                 4: ((3, NX + 1), (2, NY))}
        if int(srctype) not in boxes:
            raise ValueError(f"srctype must be 0..4, got {srctype}")
        ri, rj = boxes[int(srctype)]
    i, j = np.meshgrid(np.arange(ri[0], ri[1] + 1, dtype=np.int64),
                       np.arange(rj[0], rj[1] + 1, dtype=np.int64), indexing="ij")
    return i.reshape(-1), j.reshape(-1)


def _gauss_weights(param, x, y, sigma, i, j):
    """magn of src/Utils.jl:625-627 at 1-based cells (i, j), cell (i, j) at
    ((i-1) DELTAX, (j-1) DELTAY); also (xs - x) / (sigma DELTAX^2) and
    (ys - y) / (sigma DELTAY^2), the factors of d magn / d x and d magn / d y."""
    hx, hy = float(param.DELTAX), float(param.DELTAY)
    dx = (i - 1) * hx - float(x)
    dy = (j - 1) * hy - float(y)
    magn = 1.0 / (2 * math.pi * sigma) * np.exp(-((dx / (math.sqrt(2 * sigma) * hx)) ** 2 +
                                                 (dy / (math.sqrt(2 * sigma) * hy)) ** 2))
    return magn, dx / (sigma * hx * hx), dy / (sigma * hy * hy)


def variable_source(param, x, y, v=None, sigma=None, srctype=None, source_scale=1.0):
    """The two forms of src/Utils.jl:603-640.

    Gaussian form, variable_source(param, x, y, v; sigma): a source at every
    cell with wavelet v scaled by magn = exp(-((xs - x)^2 / (2 sigma DELTAX^2)
    + (ys - y)^2 / (2 sigma DELTAY^2))) / (2 pi sigma), xs = (i-1) DELTAX,
    ys = (j-1) DELTAY, sigma = 1 by default.  Returns (srci, srcj, srcv) with
    srcv = v magn^T of shape (len(v), ncells).  The reference covers the whole
    padded grid; the plans hold the padded frame at zero and take no sources
    there, so the cells returned are the ones a plan accepts (`srctype`
    selects the elastic field's box; None means acoustic).  The dropped frame
    terms are below magn at the frame, exp(-d^2 / (2 sigma)) / (2 pi sigma)
    for a source d cells inside it.  d loss / d (x, y, v) then follows from the
    plan's d loss / d srcv through variable_source_grad.

    Index form, variable_source(param, ix, iy; source_scale) for acoustic
    parameters: an AcousticSource at the given cells whose (NSTEP+1, n)
    wavelet is the trainable variable, zero at the start."""
    if v is None:
        from .acoustic import AcousticSource

        ix = np.asarray(x, dtype=np.int64).reshape(-1)
        iy = np.asarray(y, dtype=np.int64).reshape(-1)
        if ix.shape != iy.shape:
            raise ValueError("ix and iy differ in length")
        return AcousticSource(ix, iy, np.zeros((int(param.NSTEP) + 1, ix.size)) * source_scale)
    sigma = 1.0 if sigma is None else float(sigma)
    i, j = _source_cells(param, srctype)
    magn, _, _ = _gauss_weights(param, x, y, sigma, i, j)
    v = np.asarray(v, dtype=np.float64).reshape(-1)
    return i, j, np.ascontiguousarray(v[:, None] * magn[None, :])


def variable_source_grad(param, x, y, v, grad_srcv, sigma=None, srctype=None):
    """Chain rule of the Gaussian variable_source: from G = d loss / d srcv,
    (rows, ncells) as a plan's gradient_ex returns it for the source set
    variable_source made (rows <= len(v); rows past G's count are not
    injected), gives (d loss / d x, d loss / d y, d loss / d v):
    dv[t] = sum_k G[t, k] magn_k, dx = sum_t v[t] sum_k G[t, k] magn_k
    (xs_k - x) / (sigma DELTAX^2), and dy likewise.  G may be a numpy array or
    a torch tensor (the sums then run on its device); dv has G's kind."""
    import torch

    sigma = 1.0 if sigma is None else float(sigma)
    i, j = _source_cells(param, srctype)
    magn, fx, fy = _gauss_weights(param, x, y, sigma, i, j)
    G = torch.as_tensor(grad_srcv, dtype=torch.float64)
    if G.dim() != 2 or G.shape[1] != i.size:
        raise ValueError(f"grad_srcv has shape {tuple(G.shape)}, expected (rows, {i.size})")
    v = np.asarray(v, dtype=np.float64).reshape(-1)
    rows = G.shape[0]
    if rows > v.size:
        raise ValueError(f"grad_srcv has {rows} rows, v only {v.size}")
    W = torch.as_tensor(np.stack([magn, magn * fx, magn * fy], axis=1), device=G.device)
    P = G @ W  # (rows, 3)
    vt = torch.as_tensor(v[:rows], device=G.device)
    gx = float(vt @ P[:, 1])
    gy = float(vt @ P[:, 2])
    dv = torch.zeros(v.size, dtype=torch.float64, device=G.device)
    dv[:rows] = P[:, 0]
    if not isinstance(grad_srcv, torch.Tensor):
        dv = dv.numpy()
    return gx, gy, dv


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
