"""The autograd nodes over the plans (AcousticMisfit, ElasticMisfit): their
forward / backward wiring, composed with other torch operations, on CPU.  The
plans are replaced by stand-ins that compute with the oracle; the plans
themselves are checked against the oracle by the GPU tests."""
import numpy as np
import torch

from conftest import golden


class _AcousticOracle:
    def __init__(self, orc, NX, NY, T, dt, h, s, t, src, rcv):
        self.a = (orc, NX, NY, T, dt, h, s, t, src, rcv)

    def gradient(self, vp, observed):
        orc, NX, NY, T, dt, h, s, t, (si, sj, sv), (ri, rj) = self.a
        L, g = orc.acoustic_gradient(NX, NY, T, dt, h, h, s, t,
                                     vp.detach().numpy().reshape(-1), si, sj, sv, ri, rj,
                                     observed.numpy())
        return torch.tensor(L, dtype=torch.float64), torch.as_tensor(g).reshape(vp.shape)


class _ElasticOracle:
    def __init__(self, orc, g, T):
        self.orc, self.g, self.T = orc, g, T

    def gradient(self, lam, mu, rho, observed):
        g = self.g
        L, gl, gm, gr = self.orc.elastic_gradient(
            int(g["NX"]), int(g["NY"]), self.T, float(g["dt"]), float(g["dx"]), float(g["dy"]),
            g["ax"], g["bx"], g["ay"], g["by"], *(x.detach().numpy().astype(np.float64)
                                                  for x in (lam, mu, rho)),
            g["srci"], g["srcj"], g["srctype"], g["srcv"], g["rcvi"], g["rcvj"], g["rcvtype"],
            observed.numpy())
        return (torch.tensor(L, dtype=torch.float64),
                *(torch.as_tensor(x).reshape(lam.shape) for x in (gl, gm, gr)))


def test_acoustic_misfit_chain_rule(ads, orc):
    rng = np.random.default_rng(4)
    NX, NY, T, dt, h = 14, 12, 40, 1e-3, 10.0
    s, t = orc.acoustic_pml(NX, NY, h, h, 4, 2000.0)
    src = ([7], [6], rng.standard_normal((T, 1)) * 1e3)
    rcv = (np.arange(3, 13), np.full(10, 3))
    v0 = 2000 + 300 * rng.random((NX + 2, NY + 2))
    obs = orc.acoustic_forward(NX, NY, T, dt, h, h, s, t, (v0 * 1.03).reshape(-1), *src, *rcv)
    plan = _AcousticOracle(orc, NX, NY, T, dt, h, s, t, src, rcv)
    scale = torch.tensor(1.01, dtype=torch.float64, requires_grad=True)
    base = torch.as_tensor(v0, dtype=torch.float32).requires_grad_(True)
    vp = base * scale  # a float32 model built by torch operations
    loss = ads.AcousticMisfit.apply(vp, plan, torch.as_tensor(obs))
    (3.0 * loss).backward()
    L, g = plan.gradient(vp.detach().double(), torch.as_tensor(obs))
    assert float(loss.detach()) == float(L)
    assert base.grad.dtype == torch.float32  # the gradient comes back in the model's dtype
    assert torch.allclose(base.grad.double(), (3.0 * g * 1.01).float().double(), rtol=1e-6)
    want = float((3.0 * g * base.detach().double()).sum())
    assert abs(float(scale.grad) - want) <= 1e-5 * abs(want)  # summed in float32


def test_elastic_misfit_chain_rule(ads, orc):
    """Gradients through compute_properties (vp, vs, rho -> lambda, mu, rho)
    by autograd equal compute_properties_grad of the plan's gradients."""
    g = golden("elastic_small.npz")
    T = int(g["NSTEP"])
    plan = _ElasticOracle(orc, g, T)
    mu0 = torch.as_tensor(g["mu"])
    rho = torch.as_tensor(g["rho"]).clone().requires_grad_(True)
    vp = torch.sqrt((torch.as_tensor(g["lam"]) + 2 * mu0) / rho.detach()).requires_grad_(True)
    vs = torch.sqrt(mu0 / rho.detach()).requires_grad_(True)
    mu = rho * vs * vs
    lam = rho * vp * vp - 2 * mu
    loss = ads.ElasticMisfit.apply(lam, mu, rho, plan, torch.as_tensor(g["obs"][:, :T + 1]))
    loss.backward()
    L, gl, gm, gr = plan.gradient(lam.detach(), mu.detach(), rho.detach(),
                                  torch.as_tensor(g["obs"][:, :T + 1]))
    assert float(loss.detach()) == float(L)
    want = ads.compute_properties_grad(vp.detach(), vs.detach(), rho.detach(), gl, gm, gr)
    for got, w in zip((vp.grad, vs.grad, rho.grad), want):
        assert torch.allclose(got, w, rtol=1e-12, atol=1e-12 * w.abs().max())
