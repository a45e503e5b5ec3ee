"""FWI optimiser loop over the batched gradient (src/Optim.jl:135-192).

The reference's ``LBFGS!`` flattens the model variables, hands Optim.jl an
``f(x)`` (loss) and ``g!(G, x)`` (gradient) pair built from TF session runs,
calls ``callback(x, iter, loss)`` once per iteration and returns the loss
history.  Here the same loop runs scipy's L-BFGS-B (bounds optional) and one
plan gradient serves both the loss and the gradient at a point: the GPU does
one forward + checkpointed adjoint per function evaluation, and the plan's
CUDA graphs are replayed on every call.
"""
from __future__ import annotations

import numpy as np


def LBFGS(fg, x0, callback=None, max_iter=100, bounds=None, **options):
    """Minimise with L-BFGS-B.

    fg(x) -> (loss, grad): float64 numpy vector in, float and float64 vector out.
    callback(x, iter, loss) is called after each iteration (src/Optim.jl:182-189).
    Returns (x, losses): the final point and the loss after each iteration.
    """
    from scipy.optimize import minimize

    cache = {}

    def f(x):
        key = x.tobytes()
        if key not in cache:
            cache.clear()
            loss, g = fg(x)
            cache[key] = (float(loss), np.asarray(g, dtype=np.float64).reshape(-1))
        return cache[key]

    losses = []

    def cb(xk):
        loss = f(xk)[0]
        losses.append(loss)
        if callback is not None:
            callback(xk, len(losses), loss)

    opts = dict(maxiter=max_iter)
    opts.update(options)
    res = minimize(f, np.asarray(x0, dtype=np.float64).reshape(-1), jac=True,
                   method="L-BFGS-B", bounds=bounds, callback=cb, options=opts)
    return res.x, losses


def fwi_lbfgs(plan, vp0, observed, max_iter=20, callback=None, vmin=None, vmax=None):
    """Acoustic FWI with the parameterisation of the reference's layer-model
    example (examples/invert_velocity_model/AcousticFWI-LayerModel.jl:45-86):
    the unknown is vp / mean(vp0); loss and gradient come from
    plan.gradient (all shots, one GPU).  vmin / vmax bound vp if given.
    Returns (vp, losses)."""
    import torch

    vp0 = np.asarray(vp0, dtype=np.float64)
    shape = vp0.shape
    scale = float(vp0.mean())
    dev = observed.device
    vdev = torch.empty(shape, dtype=torch.float64, device=dev)

    def fg(x):
        vdev.copy_(torch.from_numpy(x.reshape(shape) * scale))
        loss, grad = plan.gradient(vdev, observed)
        return float(loss), grad.cpu().numpy().reshape(-1) * scale

    bounds = None
    if vmin is not None or vmax is not None:
        lo = -np.inf if vmin is None else vmin / scale
        hi = np.inf if vmax is None else vmax / scale
        bounds = [(lo, hi)] * vp0.size
    x, losses = LBFGS(fg, vp0.reshape(-1) / scale, callback=callback, max_iter=max_iter,
                      bounds=bounds)
    return x.reshape(shape) * scale, losses



def source_objective(plan, param, vp, observed, sigma=0.5, source_scale=1.0, shot=0):
    """The objective of the reference's source location and wavelet inversion
    (examples/invert_source_location_time_function/AcousticFWI-LayerModel-Source.jl):
    unknowns z = (a, b, w) with x = sigmoid(a) DELTAX NX, y = sigmoid(b)
    DELTAY NY and wavelet v = w source_scale; the source is the Gaussian
    variable_source(param, x, y, v; sigma).

    `plan` is an AcousticPlan whose shot `shot` was created with the cells of
    that source (variable_source's srci / srcj, which do not depend on x, y,
    v) and whose window `param` describes (NX = nx, NY = MY, NSTEP = nstep).
    Returns (fg, unpack): fg(z) -> (loss, d loss / d z) writes v magn^T into
    the plan on the device (set_source_values), runs one gradient with
    d loss / d srcv and applies variable_source_grad and the sigmoid chain
    rule (the model vp stays fixed); unpack(z) -> (x, y, v)."""
    import torch

    from .utils import _gauss_weights, _source_cells, variable_source_grad

    sig = float(sigma)
    Lx, Ly = param.DELTAX * param.NX, param.DELTAY * param.NY
    i, j = _source_cells(param, None)
    dev = observed.device

    def parts(z):
        sa, sb = 1 / (1 + np.exp(-z[0])), 1 / (1 + np.exp(-z[1]))
        return sa, sb, sa * Lx, sb * Ly, np.asarray(z[2:], dtype=np.float64) * source_scale

    def fg(z):
        sa, sb, x, y, v = parts(z)
        magn, _, _ = _gauss_weights(param, x, y, sig, i, j)
        srcv = (torch.as_tensor(v, device=dev)[:, None] *
                torch.as_tensor(magn, device=dev)[None, :])
        plan.set_source_values(shot, srcv)
        loss, _, gs = plan.gradient(vp, observed, want_source_grad=True)
        gx, gy, gv = variable_source_grad(param, x, y, v, gs[shot], sigma=sig)
        gv = gv.cpu().numpy() if isinstance(gv, torch.Tensor) else gv
        g = np.concatenate([[gx * Lx * sa * (1 - sa), gy * Ly * sb * (1 - sb)],
                            gv * source_scale])
        return float(loss), g

    def unpack(z):
        return parts(z)[2:]

    return fg, unpack


def source_lbfgs(plan, param, vp, observed, x0, y0, v0, sigma=0.5, source_scale=1.0, shot=0,
                 max_iter=20, callback=None):
    """L-BFGS over source_objective from the source position (x0, y0) and
    wavelet v0 (length >= NSTEP).  The optimiser sees the loss divided by its
    starting value, so its stopping tolerances are relative; the callback and
    the returned history carry the loss itself.  Returns (x, y, v, losses)."""
    fg, unpack = source_objective(plan, param, vp, observed, sigma, source_scale, shot)
    Lx, Ly = param.DELTAX * param.NX, param.DELTAY * param.NY

    def logit(p):
        return float(np.log(p / (1 - p)))

    z0 = np.concatenate([[logit(x0 / Lx), logit(y0 / Ly)],
                         np.asarray(v0, dtype=np.float64).reshape(-1) / source_scale])
    L0 = fg(z0)[0]
    scale = 1.0 / L0 if L0 > 0 else 1.0

    def fgn(z):
        loss, g = fg(z)
        return loss * scale, g * scale

    cb = None if callback is None else (lambda z, it, loss: callback(z, it, loss / scale))
    z, losses = LBFGS(fgn, z0, callback=cb, max_iter=max_iter)
    x, y, v = unpack(z)
    return x, y, v, [l / scale for l in losses]


def wavelet_lbfgs(plan, model, observed, v0, source_scale=1.0, shot=0, max_iter=20,
                  callback=None):
    """Wavelet (rupture-process) inversion with the parameterisation of the
    reference's example (examples/invert_rupture_process/AcousticFWI-LayerModel-Rupture.jl):
    the unknown is shot `shot`'s wavelet matrix w, srcv = w source_scale, as
    variable_source's index form (src/Utils.jl:636-640) makes it trainable.

    `plan` is an AcousticPlan (model = vp) or an ElasticPlan created with
    source_gradient (model = (lambda, mu, rho)); v0 is the starting srcv,
    (rows, nsrc) with rows >= the shot's step count.  Every evaluation writes
    srcv into the plan (set_source_values) and takes d loss / d srcv from one
    gradient; rows the plan never injects have a zero gradient.  The
    optimiser sees the loss divided by its starting value.  Returns
    (srcv, losses)."""
    import torch

    model = (model,) if isinstance(model, torch.Tensor) else tuple(model)
    v0 = np.asarray(v0, dtype=np.float64)
    shape = v0.shape
    dev = observed.device

    def fg(z):
        srcv = torch.as_tensor(z.reshape(shape) * source_scale, device=dev)
        plan.set_source_values(shot, srcv)
        out = plan.gradient(*model, observed, want_source_grad=True)
        G = out[-1][shot]
        g = np.zeros(shape)
        g[:G.shape[0]] = G.cpu().numpy()
        return float(out[0]), g.reshape(-1) * source_scale

    z0 = v0.reshape(-1) / source_scale
    L0 = fg(z0)[0]
    scale = 1.0 / L0 if L0 > 0 else 1.0

    def fgn(z):
        loss, g = fg(z)
        return loss * scale, g * scale

    cb = None if callback is None else (lambda z, it, loss: callback(z, it, loss / scale))
    z, losses = LBFGS(fgn, z0, callback=cb, max_iter=max_iter)
    return z.reshape(shape) * source_scale, [l / scale for l in losses]
