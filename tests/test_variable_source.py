"""The Gaussian variable source (src/Utils.jl:603-633) and its location
gradient: variable_source's cells and weights, and variable_source_grad's
chain rule from d loss / d srcv (computed here by the oracle's adjoint)
against central differences of the oracle's loss in x, y and v."""
import math

import numpy as np
import pytest

from conftest import golden


def _reference_magn(p, x, y, sigma, i, j):
    """magn exactly as src/Utils.jl:625-627 writes it, at 1-based cells."""
    xs, ys = (i - 1) * p.DELTAX, (j - 1) * p.DELTAY
    return 1 / (2 * math.pi * sigma) * np.exp(-(((xs - x) / (math.sqrt(2 * sigma) * p.DELTAX)) ** 2 +
                                               ((ys - y) / (math.sqrt(2 * sigma) * p.DELTAY)) ** 2))


def test_cells_weights_and_index_form(ads):
    p = ads.AcousticPropagatorParams(NX=12, NY=9, NSTEP=30, DELTAX=10.0, DELTAY=8.0)
    v = np.linspace(-1, 2, 30)
    i, j, srcv = ads.variable_source(p, 55.0, 41.0, v, sigma=1.5)
    assert i.size == 12 * 9 and i.min() == 2 and i.max() == 13 and j.min() == 2 and j.max() == 10
    assert np.array_equal(i[:9], np.full(9, 2)) and np.array_equal(j[:9], np.arange(2, 11))
    m = _reference_magn(p, 55.0, 41.0, 1.5, i, j)
    assert srcv.shape == (30, i.size) and np.allclose(srcv, v[:, None] * m[None], rtol=1e-15)
    e = ads.ElasticPropagatorParams(NX=12, NY=9, NSTEP=30)
    for t, (ri, rj) in {0: ((3, 13), (3, 10)), 1: ((2, 12), (2, 9)), 2: ((2, 12), (3, 10)),
                        3: ((2, 12), (3, 10)), 4: ((3, 13), (2, 9))}.items():
        i, j, _ = ads.variable_source(e, 40.0, 30.0, v, srctype=t)
        assert (i.min(), i.max(), j.min(), j.max()) == (ri[0], ri[1], rj[0], rj[1])
        assert i.size == (ri[1] - ri[0] + 1) * (rj[1] - rj[0] + 1)
    with pytest.raises(ValueError):
        ads.variable_source(e, 40.0, 30.0, v, srctype=7)
    src = ads.variable_source(p, [4, 5], [6, 7], source_scale=2.0)
    assert src.srcv.shape == (31, 2) and np.all(src.srcv == 0)
    assert list(src.srci) == [4, 5] and list(src.srcj) == [6, 7]


def test_acoustic_location_gradient_finite_differences(ads, orc):
    rng = np.random.default_rng(11)
    p = ads.AcousticPropagatorParams(NX=20, NY=16, NSTEP=40, DELTAX=10.0, DELTAY=10.0,
                                     DELTAT=1e-3)
    NX, NY, T = p.NX, p.NY, p.NSTEP
    N = (NX + 2) * (NY + 2)
    vp = 2000 + 500 * rng.random(N)
    s, t = orc.acoustic_pml(NX, NY, 10.0, 10.0, 5, 2000.0)
    rcvi, rcvj = np.arange(3, 19), np.full(16, 3)
    v = ads.Ricker(p, 4.0, 12.0) * 1e3
    x, y, sig = 103.0, 86.0, 1.3

    def loss(x, y, v, want=False):
        i, j, srcv = ads.variable_source(p, x, y, v, sigma=sig)
        return orc.acoustic_gradient(NX, NY, T, p.DELTAT, 10.0, 10.0, s, t, vp, i, j, srcv,
                                     rcvi, rcvj, obs, want_src=want)

    i0, j0, sv0 = ads.variable_source(p, x + 21.0, y - 17.0, v, sigma=sig)
    obs = orc.acoustic_forward(NX, NY, T, p.DELTAT, 10.0, 10.0, s, t, vp * 1.02, i0, j0, sv0,
                               rcvi, rcvj)
    L, _, G = loss(x, y, v, True)
    gx, gy, gv = ads.variable_source_grad(p, x, y, v, G, sigma=sig)
    e = 1e-3
    fx = (loss(x + e, y, v)[0] - loss(x - e, y, v)[0]) / (2 * e)
    fy = (loss(x, y + e, v)[0] - loss(x, y - e, v)[0]) / (2 * e)
    assert abs(fx - gx) <= 1e-6 * abs(fx) and abs(fy - gy) <= 1e-6 * abs(fy), (fx, gx, fy, gy)
    assert gv.shape == v.shape and gv[0] == 0.0  # row 0 is never injected
    for k in (5, 17, T - 1):
        vp_, vm_ = v.copy(), v.copy()
        vp_[k] += 1.0
        vm_[k] -= 1.0
        fv = (loss(x, y, vp_)[0] - loss(x, y, vm_)[0]) / 2.0
        assert abs(fv - gv[k]) <= 1e-7 * abs(fv) + 1e-15 * L, (k, fv, gv[k])


def test_elastic_location_gradient_finite_differences(ads, orc):
    g = golden("elastic_small.npz")
    NX, NY, T = int(g["NX"]), int(g["NY"]), 30
    p = ads.ElasticPropagatorParams(NX=NX, NY=NY, NSTEP=T, DELTAX=float(g["dx"]),
                                    DELTAY=float(g["dy"]), DELTAT=float(g["dt"]))
    v = np.random.default_rng(12).standard_normal(T) * 1e6
    x, y, st = 131.0, 97.0, 3

    def loss(x, y, want=False):
        i, j, srcv = ads.variable_source(p, x, y, v, srctype=st)
        return orc.elastic_gradient(NX, NY, T, p.DELTAT, p.DELTAX, p.DELTAY, g["ax"], g["bx"],
                                    g["ay"], g["by"], g["lam"], g["mu"], g["rho"], i, j,
                                    np.full(i.size, st), srcv, g["rcvi"], g["rcvj"],
                                    g["rcvtype"], g["obs"][:, :T + 1], want_src=want)

    out = loss(x, y, True)
    gx, gy, gv = ads.variable_source_grad(p, x, y, v, out[4], srctype=st)
    e = 1e-3
    fx = (loss(x + e, y)[0] - loss(x - e, y)[0]) / (2 * e)
    fy = (loss(x, y + e)[0] - loss(x, y - e)[0]) / (2 * e)
    assert abs(fx - gx) <= 1e-6 * abs(fx) and abs(fy - gy) <= 1e-6 * abs(fy), (fx, gx, fy, gy)
    assert gv.shape == v.shape


class _OraclePlan:
    """A CPU stand-in for an acoustic plan with one shot, computed by the
    oracle: the two calls source_objective makes (set_source_values and
    gradient with d loss / d srcv)."""

    def __init__(self, orc, p, sig, tau, vp, i, j, rcvi, rcvj):
        self.orc, self.p, self.sig, self.tau = orc, p, sig, tau
        self.i, self.j, self.rcvi, self.rcvj = i, j, rcvi, rcvj
        self.srcv = None

    def set_source_values(self, shot, srcv):
        assert shot == 0
        self.srcv = srcv.cpu().numpy()[:self.p.NSTEP]

    def gradient(self, vp, observed, want_source_grad=False):
        import torch

        p = self.p
        L, g, G = self.orc.acoustic_gradient(p.NX, p.NY, p.NSTEP, p.DELTAT, p.DELTAX, p.DELTAY,
                                             self.sig, self.tau, vp.numpy().reshape(-1),
                                             self.i, self.j, self.srcv, self.rcvi, self.rcvj,
                                             observed.numpy(), want_src=True)
        return torch.tensor(L, dtype=torch.float64), torch.as_tensor(g), [torch.as_tensor(G)]


def _source_case(ads, orc):
    import torch

    rng = np.random.default_rng(21)
    p = ads.AcousticPropagatorParams(NX=20, NY=16, NSTEP=60, DELTAX=10.0, DELTAY=10.0,
                                     DELTAT=1e-3)
    vp = 2000 + 300 * rng.random((p.NX + 2) * (p.NY + 2))
    s, t = orc.acoustic_pml(p.NX, p.NY, 10.0, 10.0, 4, 2000.0)
    rcvi, rcvj = np.arange(3, 21), np.full(18, 3)
    v = ads.Ricker(p, 3.0, 10.0)
    i, j, sv = ads.variable_source(p, 103.0, 86.0, v * 1e3, sigma=0.5)
    obs = orc.acoustic_forward(p.NX, p.NY, p.NSTEP, p.DELTAT, 10.0, 10.0, s, t, vp, i, j, sv,
                               rcvi, rcvj)
    plan = _OraclePlan(orc, p, s, t, vp, i, j, rcvi, rcvj)
    return p, plan, torch.as_tensor(vp), torch.as_tensor(obs), v


def test_source_objective_gradient_finite_differences(ads, orc):
    """d loss / d (a, b, w) of the source inversion objective (sigmoid
    position, scaled wavelet) against central differences."""
    p, plan, vp, obs, v = _source_case(ads, orc)
    fg, unpack = ads.source_objective(plan, p, vp, obs, sigma=0.5, source_scale=1e3)
    z = np.concatenate([[0.3, 0.1], 0.9 * v])
    L, g = fg(z)
    x, y, vv = unpack(z)
    assert abs(x - 200 / (1 + np.exp(-0.3))) < 1e-12 and np.allclose(vv, 0.9e3 * v)
    for k, e in [(0, 1e-5), (1, 1e-5), (12, 1e-3), (30, 1e-3)]:
        zp, zm = z.copy(), z.copy()
        zp[k] += e
        zm[k] -= e
        fd = (fg(zp)[0] - fg(zm)[0]) / (2 * e)
        assert abs(fd - g[k]) <= 1e-6 * abs(fd) + 1e-12 * L, (k, fd, g[k])


def test_source_lbfgs_recovers_location(ads, orc):
    """The inversion loop moves a misplaced Gaussian source back onto the
    one that made the data (wavelet known up to a 20% scale)."""
    p, plan, vp, obs, v = _source_case(ads, orc)
    x, y, vv, losses = ads.source_lbfgs(plan, p, vp, obs, 116.0, 77.0, 0.8 * v, sigma=0.5,
                                        source_scale=1e3, max_iter=25)
    err0 = np.hypot(116.0 - 103.0, 77.0 - 86.0)
    assert losses[-1] < 1e-3 * losses[0], losses
    assert np.hypot(x - 103.0, y - 86.0) < 0.05 * err0, (x, y)


def test_wavelet_lbfgs_fits_the_rupture_wavelets(ads, orc):
    """The rupture-process inversion loop (index-form variable source, all
    wavelets unknown, starting from zero) on the oracle stand-in: the misfit
    falls by orders of magnitude and the unused rows keep a zero gradient."""
    import torch

    rng = np.random.default_rng(5)
    p = ads.AcousticPropagatorParams(NX=20, NY=16, NSTEP=50, DELTAX=10.0, DELTAY=10.0,
                                     DELTAT=1e-3)
    vp = 2000 + 300 * rng.random((p.NX + 2) * (p.NY + 2))
    s, t = orc.acoustic_pml(p.NX, p.NY, 10.0, 10.0, 4, 2000.0)
    rcvi, rcvj = np.arange(3, 21), np.full(18, 3)
    src = ads.variable_source(p, [8, 10, 12, 14], [12, 12, 12, 12], source_scale=1e3)
    assert src.srcv.shape == (51, 4)
    true = np.stack([np.roll(ads.Ricker(p, 3.0, 10.0), 3 * k) for k in range(4)], axis=1)
    true = np.vstack([true, np.zeros((1, 4))]) * 1e3
    obs = orc.acoustic_forward(p.NX, p.NY, p.NSTEP, p.DELTAT, 10.0, 10.0, s, t, vp, src.srci,
                               src.srcj, true, rcvi, rcvj)
    plan = _OraclePlan(orc, p, s, t, vp, src.srci, src.srcj, rcvi, rcvj)
    seen = []
    w, losses = ads.wavelet_lbfgs(plan, torch.as_tensor(vp), torch.as_tensor(obs), src.srcv,
                                  source_scale=1e3, max_iter=30,
                                  callback=lambda z, it, loss: seen.append(loss))
    assert w.shape == (51, 4) and len(seen) == len(losses) and seen == losses
    assert losses[-1] < 1e-2 * losses[0], losses
    assert np.all(w[-1] == 0.0)  # row NSTEP is never injected: its gradient is zero
