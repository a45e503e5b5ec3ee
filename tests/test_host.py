"""Host-side logic: wavelets and material transforms against the reference
formulas, synthetic model generators, parameter defaults."""
import math

import numpy as np
import pytest


def test_ricker_matches_formula(ads):
    p = ads.AcousticPropagatorParams(NSTEP=300, DELTAT=1e-3)
    a, shift = ads.ricker_width_samples(10.0, 1e-3), 150.0
    w = ads.Ricker(p, a, shift, 2.0)
    x = np.arange(1, 301) - shift
    A = 2 / (math.sqrt(3 * a) * math.pi ** 0.25)
    ref = 2.0 * A * (1 - x ** 2 / a ** 2) * np.exp(-x ** 2 / (2 * a ** 2))
    assert np.allclose(w, ref, rtol=1e-14, atol=0)
    assert np.argmax(w) == 149


def test_material_transforms(ads):
    vp, vs, rho = np.array([3000.0]), np.array([1700.0]), np.array([2200.0])
    lam, mu, r = ads.compute_properties(vp, vs, rho)
    assert mu[0] == 2200.0 * 1700.0 * 1700.0
    assert lam[0] == 2200.0 * 3000.0 * 3000.0 - 2 * mu[0]
    lam2, mu2, _ = ads.compute_lame_parameters(vp, vs, rho)
    assert np.allclose(lam2, lam) and np.allclose(mu2, mu)
    lg, mg, rg = ads.compute_lame_parameters(4, 3, 3300.0, 3300.0 / 1.732, 2800.0)
    assert lg.shape == mg.shape == rg.shape == (6, 5) and np.all(rg == 2800.0)
    assert np.all(mg == 2800.0 * (3300.0 / 1.732) ** 2)
    assert np.all(lg == 2800.0 * (3300.0 ** 2 - 2.0 * (3300.0 / 1.732) ** 2))


def test_properties_chain_rule_matches_finite_differences(ads):
    """d L / d (vp, vs, rho) for L = <a, lambda> + <b, mu> + <c, rho> through
    compute_properties, against central differences."""
    rng = np.random.default_rng(2)
    vp = 2500 + 1000 * rng.random(6)
    vs = vp / np.sqrt(3) * (1 + 0.05 * rng.standard_normal(6))
    rho = 310 * vp ** 0.25
    a, b, c = rng.standard_normal((3, 6))

    def L(vp, vs, rho):
        lam, mu, r = ads.compute_properties(vp, vs, rho)
        return a @ lam + b @ mu + c @ r

    g = ads.compute_properties_grad(vp, vs, rho, a, b, c)
    for k, x in enumerate((vp, vs, rho)):
        for m in range(6):
            e = 1e-3 * x[m]
            xp, xm = x.copy(), x.copy()
            xp[m] += e
            xm[m] -= e
            args_p = [xp if q == k else y for q, y in enumerate((vp, vs, rho))]
            args_m = [xm if q == k else y for q, y in enumerate((vp, vs, rho))]
            fd = (L(*args_p) - L(*args_m)) / (2 * e)
            assert abs(fd - g[k][m]) <= 1e-7 * max(abs(fd), 1e-3 * np.abs(g[k]).max()), (k, m)


def test_gradtest_orders(ads, orc):
    """gradtest on the oracle's acoustic loss and gradient (a small case):
    the first-order difference falls as O(gamma), the Taylor remainder with
    the adjoint gradient as O(gamma^2); a wrong gradient stays O(gamma)."""
    rng = np.random.default_rng(3)
    NX, NY, T = 16, 12, 40
    s, t = orc.acoustic_pml(NX, NY, 10.0, 10.0, 4, 2000.0)
    vp0 = 2000 + 300 * rng.random((NX + 2) * (NY + 2))
    srcv = rng.standard_normal((T, 1)) * 1e3
    rcvi, rcvj = np.arange(3, 15), np.full(12, 3)
    obs = orc.acoustic_forward(NX, NY, T, 1e-3, 10.0, 10.0, s, t, vp0 * 1.02, [9], [7], srcv,
                               rcvi, rcvj)

    def fg(vp):
        return orc.acoustic_gradient(NX, NY, T, 1e-3, 10.0, 10.0, s, t, vp, [9], [7], srcv,
                                     rcvi, rcvj, obs)

    g, S, W = ads.gradtest(fg, vp0, direction=rng.random(vp0.size) * 10.0)
    assert np.allclose(g, [1e-1, 1e-2, 1e-3, 1e-4, 1e-5])
    assert all(1 / 12 < abs(S[k + 1] / S[k]) < 1 / 8 for k in range(4))
    assert all(abs(W[k + 1] / W[k]) < 1 / 50 for k in range(3))
    _, _, W2 = ads.gradtest(lambda v: (fg(v)[0], fg(v)[1] * 1.1), vp0,
                            direction=rng.random(vp0.size) * 10.0)
    assert abs(W2[3] / W2[2]) > 1 / 12


def test_add_initial_model_centres_the_update(ads):
    v = np.zeros((6, 8))
    out = ads.add_initial_model(np.ones((2, 4)), v)
    assert out.sum() == 8 and np.all(out[2:4, 2:6] == 1)
    stack = ads.add_initial_model(np.ones((3, 2, 2)), v)
    assert stack.shape == (3, 6, 8) and np.all(stack[:, 2:4, 3:5] == 1)
    big = np.arange(10 * 12, dtype=float).reshape(10, 12)
    assert np.array_equal(ads.add_initial_model(big, v), big[2:8, 2:10])
    with pytest.raises(ValueError):
        ads.add_initial_model(np.ones((8, 2)), v)


def test_param_defaults_follow_reference(ads):
    a = ads.AcousticPropagatorParams()
    assert (a.NX, a.NY, a.NSTEP, a.NPOINTS_PML, a.vp_ref, a.Rcoef) == (101, 641, 4000, 12, 1000.0, 0.001)
    e = ads.ElasticPropagatorParams(f0=5.0)
    assert e.ALPHA_MAX_PML == 2 * math.pi * 2.5 and e.vp_ref == 2000.0 and e.K_MAX_PML == 1.0
    assert a.use_pml == 15


def test_models_are_seeded(ads):
    a = ads.folded_layer_model(100, 50, seed=3)
    b = ads.folded_layer_model(100, 50, seed=3)
    assert np.array_equal(a, b) and a.min() >= 1500 and a.max() <= 4500
    v = ads.layered_gaussian_model(60, 60, seed=1)
    assert v.shape == (60, 60) and 1700 < v.min() < v.max() < 4000


def test_lbfgs_driver_quadratic():
    """The L-BFGS loop (f/g from one call, callback(x, iter, loss), loss history)
    on a convex quadratic: reaches the minimiser."""
    import pytest

    pytest.importorskip("scipy")
    import __graft_entry__ as g

    pkg = g.load_package()
    rng = np.random.default_rng(0)
    A = rng.standard_normal((12, 12))
    H = A @ A.T + 12 * np.eye(12)
    b = rng.standard_normal(12)
    calls = []

    def fg(x):
        calls.append(1)
        return 0.5 * x @ H @ x - b @ x, H @ x - b

    seen = []
    x, losses = pkg.LBFGS(fg, np.zeros(12), callback=lambda x, it, l: seen.append((it, l)),
                          max_iter=200, ftol=1e-15, gtol=1e-12)
    assert np.allclose(x, np.linalg.solve(H, b), rtol=1e-6, atol=1e-8)
    assert len(losses) == len(seen) and [s[0] for s in seen] == list(range(1, len(seen) + 1))
    assert all(losses[k + 1] <= losses[k] + 1e-12 for k in range(len(losses) - 1))
