"""Host-side logic: wavelets and material transforms against the reference
formulas, synthetic model generators, parameter defaults."""
import math

import numpy as np


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
