"""The real-model fixture through the GPU path: the reference's Marmousi2 FWI
example (examples/nn_fwi/FWI_inversion.jl: load_params(model, vp_ref=1e3),
load_acoustic_source / load_acoustic_receiver, compute_loss_and_grads_GPU),
8 shots x 183 receivers on the 202 x 68 model, 1678 steps, loaded by the
package's MAT loaders from tests/golden/marmousi2_fwi.mat.  The FP64 plans
match the oracle to rel-L2 <= 1e-12 (traces, loss, gradient)."""
import os

import numpy as np
import pytest
import torch

from conftest import ROOT

pytestmark = pytest.mark.gpu

FIX = os.path.join(ROOT, "tests", "golden", "marmousi2_fwi.mat")
TOL64 = 1e-12


def rel(a, b):
    a, b = np.asarray(a, dtype=np.float64), np.asarray(b, dtype=np.float64)
    return float(np.linalg.norm(a - b) / max(np.linalg.norm(b), 1e-300))


@pytest.fixture(scope="module")
def marmousi(ads, orc):
    from scipy.io import loadmat

    p = ads.load_params(FIX, vp_ref=1e3, PropagatorKernel=1)
    vp0 = ads.load_acoustic_model(FIX).vp
    vpt = np.asarray(loadmat(FIX)["vp_true"], dtype=np.float64)
    srcs, rcvs = ads.load_acoustic_source(FIX), ads.load_acoustic_receiver(FIX)
    sx, ty = orc.acoustic_pml(p.NX, p.NY, p.DELTAX, p.DELTAY, p.NPOINTS_PML, p.vp_ref)
    return p, vp0, vpt, srcs, rcvs, sx, ty


def _fwd(orc, p, sx, ty, vp, s, r, variant):
    return orc.acoustic_forward(p.NX, p.NY, p.NSTEP, p.DELTAT, p.DELTAX, p.DELTAY, sx, ty,
                                vp.reshape(-1), s.srci, s.srcj, s.srcv, r.rcvi, r.rcvj,
                                variant=variant)


@pytest.mark.parametrize("kernel", [1, 0])
def test_marmousi_forward_and_gradient_fp64(ads, orc, cuda, marmousi, kernel):
    """PropagatorKernel 1 (the custom operators' form) and 0 (the reference's
    default one_step form, phi / psi from the new u)."""
    p, vp0, vpt, srcs, rcvs, sx, ty = marmousi
    p.PropagatorKernel = kernel
    variant = 0 if kernel == 1 else 1  # oracle: 0 = w form, 1 = u form
    assert len(srcs) == 8 and all(len(r.rcvi) == 183 for r in rcvs)
    obs = [_fwd(orc, p, sx, ty, vpt, s, r, variant) for s, r in zip(srcs, rcvs)]
    got = ads.compute_forward_GPU(p, srcs, rcvs, vpt)
    assert max(rel(g.cpu().numpy(), o) for g, o in zip(got, obs)) <= TOL64
    loss, grad = ads.compute_loss_and_grads_GPU(p, srcs, rcvs, obs, vp0)
    lref, gref = 0.0, 0.0
    for s, r, o in zip(srcs, rcvs, obs):
        l, g = orc.acoustic_gradient(p.NX, p.NY, p.NSTEP, p.DELTAT, p.DELTAX, p.DELTAY, sx, ty,
                                     vp0.reshape(-1), s.srci, s.srcj, s.srcv, r.rcvi, r.rcvj,
                                     o, variant=variant)
        lref, gref = lref + l, gref + g
    assert abs(float(loss) - lref) <= TOL64 * lref
    assert rel(torch.as_tensor(grad).cpu().numpy().reshape(-1), gref) <= TOL64
