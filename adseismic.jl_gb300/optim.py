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
