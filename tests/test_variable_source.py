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
