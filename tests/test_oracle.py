"""The oracle pinned against the reference: golden vectors produced by the
reference's own compiled CPU operators (tests/golden), the compiled reference
itself when its checkout is present, finite differences and adjoint identities."""
import numpy as np
import pytest

from conftest import golden


def test_acoustic_step_matches_reference_bitwise(orc):
    g = golden("acoustic_step.npz")
    NX, NY = int(g["NX"]), int(g["NY"])
    args = [g[k] for k in ("w", "wold", "phi", "psi", "sigma", "tau", "c")]
    u, po, qo = orc.acoustic_step_fwd(*args, float(g["dt"]), float(g["hx"]), float(g["hy"]),
                                      NX, NY)
    assert np.array_equal(u, g["u"]) and np.array_equal(po, g["phiout"])
    assert np.array_equal(qo, g["psiout"])
    grads = orc.acoustic_step_bwd(g["grad_u"], g["grad_phiout"], g["grad_psiout"], *args,
                                  float(g["dt"]), float(g["hx"]), float(g["hy"]), NX, NY,
                                  g["u"], g["phiout"], g["psiout"])
    for got, key in zip(grads, ("grad_w", "grad_wold", "grad_phi", "grad_psi", "grad_c")):
        assert np.array_equal(got, g[key]), key


def test_acoustic_loop_and_gradient_match_reference(orc):
    g = golden("acoustic_loop.npz")
    NX, NY, T = int(g["NX"]), int(g["NY"]), int(g["NSTEP"])
    dt, h = float(g["dt"]), float(g["h"])
    s, t = orc.acoustic_pml(NX, NY, h, h, int(g["npml"]), float(g["vp_ref"]))
    assert np.array_equal(s, g["sigma"]) and np.array_equal(t, g["tau"])
    rcvv = orc.acoustic_forward(NX, NY, T, dt, h, h, s, t, g["vp"], g["srci"], g["srcj"],
                                g["srcv"], g["rcvi"], g["rcvj"])
    assert np.array_equal(rcvv, g["rcvv"])
    loss, grad = orc.acoustic_gradient(NX, NY, T, dt, h, h, s, t, g["vp"], g["srci"],
                                       g["srcj"], g["srcv"], g["rcvi"], g["rcvj"], g["obs"])
    assert loss == pytest.approx(float(g["loss"]), rel=1e-14)
    assert np.linalg.norm(grad - g["grad_vp"]) <= 1e-13 * np.linalg.norm(g["grad_vp"])


def test_index_ops_match_reference(orc):
    g = golden("index_ops.npz")
    NX, NY = int(g["NX"]), int(g["NY"])
    out5 = orc.add_source_fwd(g["in5"], g["srci"], g["srcj"], g["srctype"], g["srcv"], NX, NY)
    assert np.array_equal(out5, g["out5"])
    gin5, gs = orc.add_source_bwd(g["g5"], g["srci"], g["srcj"], g["srctype"], NX, NY)
    assert np.array_equal(gin5, g["gin5"]) and np.array_equal(gs, g["grad_srcv"])
    rec = orc.get_receive_fwd(list(g["f5"]), g["rcvi"], g["rcvj"], g["rcvtype"], NX, NY)
    assert np.array_equal(rec, g["rec"])
    grec = orc.get_receive_bwd(g["gout"], int(g["nt"]), g["rcvi"], g["rcvj"], g["rcvtype"],
                               NX, NY)
    for a, b in zip(grec, g["grec"]):
        assert np.array_equal(a, b)


@pytest.mark.skipif(not __import__("oracle").ref_available(),
                    reason="compiled reference (oracle/_ref) not built here")
def test_restatement_equals_compiled_reference_random(orc):
    rng = np.random.default_rng(99)
    for NX, NY in ((1, 1), (3, 7), (17, 5)):
        N = (NX + 2) * (NY + 2)
        args = [rng.standard_normal(N) for _ in range(7)]
        a = orc.acoustic_step_fwd(*args, 0.3, 0.7, 1.1, NX, NY)
        b = orc.acoustic_step_fwd(*args, 0.3, 0.7, 1.1, NX, NY, use_ref=True)
        assert all(np.array_equal(x, y) for x, y in zip(a, b))
        g = [rng.standard_normal(N) for _ in range(3)]
        a2 = orc.acoustic_step_bwd(*g, *args, 0.3, 0.7, 1.1, NX, NY, *a)
        b2 = orc.acoustic_step_bwd(*g, *args, 0.3, 0.7, 1.1, NX, NY, *a, use_ref=True)
        assert all(np.array_equal(x, y) for x, y in zip(a2, b2))


@pytest.mark.parametrize("variant", [0, 1])
def test_acoustic_gradient_finite_differences(orc, variant):
    rng = np.random.default_rng(2)
    NX, NY, T = 20, 16, 50
    N = (NX + 2) * (NY + 2)
    dt, h = 1e-3, 10.0
    vp = 2000 + 500 * rng.random(N)
    s, t = orc.acoustic_pml(NX, NY, h, h, 5, 2000.0)
    srci, srcj, srcv = [11], [6], rng.standard_normal((T, 1)) * 1e3
    rcvi, rcvj = np.arange(3, 19), np.full(16, 3)
    obs = orc.acoustic_forward(NX, NY, T, dt, h, h, s, t, vp * 1.03, srci, srcj, srcv, rcvi,
                               rcvj, variant=variant)
    _, g = orc.acoustic_gradient(NX, NY, T, dt, h, h, s, t, vp, srci, srcj, srcv, rcvi,
                                 rcvj, obs, variant=variant)
    for cell in [(8, 6), (11, 4), (15, 9)]:
        x = cell[0] * (NY + 2) + cell[1]
        e = 1e-4 * vp[x]
        lp = orc.acoustic_gradient(NX, NY, T, dt, h, h, s, t, _bump(vp, x, e), srci, srcj,
                                   srcv, rcvi, rcvj, obs, variant=variant)[0]
        lm = orc.acoustic_gradient(NX, NY, T, dt, h, h, s, t, _bump(vp, x, -e), srci, srcj,
                                   srcv, rcvi, rcvj, obs, variant=variant)[0]
        fd = (lp - lm) / (2 * e)
        assert abs(fd - g[x]) <= 1e-6 * abs(fd) + 1e-30, (cell, fd, g[x])


def _bump(a, x, e):
    b = a.copy()
    b[x] += e
    return b


def test_variant_u_step_adjoint_identity(orc):
    rng = np.random.default_rng(4)
    NX, NY = 9, 13
    N = (NX + 2) * (NY + 2)
    sig, tau, c = rng.random(N), rng.random(N), rng.random(N)
    f = lambda x: orc.acoustic_step_fwd(x[0], x[1], x[2], x[3], sig, tau, c, 0.1, 0.2, 0.3,
                                        NX, NY, variant=1)
    v = [rng.standard_normal(N) for _ in range(4)]
    w = [rng.standard_normal(N) for _ in range(3)]
    Jv = f(v)
    gs = orc.acoustic_step_bwd(*w, *v, sig, tau, c, 0.1, 0.2, 0.3, NX, NY, *Jv, variant=1)
    lhs = sum(np.dot(a, b) for a, b in zip(Jv, w))
    rhs = sum(np.dot(a, b) for a, b in zip(gs[:4], v))
    assert abs(lhs - rhs) <= 1e-12 * abs(lhs)


def test_elastic_adjoint_identity_and_parameter_derivatives(orc):
    g = golden("elastic_small.npz")
    NX, NY = int(g["NX"]), int(g["NY"])
    N = (NX + 2) * (NY + 2)
    dt, dx, dy = float(g["dt"]), float(g["dx"]), float(g["dy"])
    lam, mu, rho = g["lam"], g["mu"], g["rho"]
    ax, bx, ay, by = g["ax"], g["bx"], g["ay"], g["by"]
    rng = np.random.default_rng(8)
    st, v, w = (rng.standard_normal(13 * N) for _ in range(3))
    Jv = orc.elastic_step_fwd(v, lam, mu, rho, ax, bx, ay, by, dt, dx, dy, NX, NY)
    gin, gl, gm, gr = orc.elastic_step_bwd(st, w, lam, mu, rho, ax, bx, ay, by, dt, dx, dy,
                                           NX, NY)
    assert abs(np.dot(Jv, w) - np.dot(v, gin)) <= 1e-13 * abs(np.dot(Jv, w))
    for name, G in (("lam", gl), ("mu", gm), ("rho", gr)):
        P = dict(lam=lam, mu=mu, rho=rho)
        dP = rng.standard_normal(N) * P[name] * 1e-6
        Pp, Pm = dict(P), dict(P)
        Pp[name] = P[name] + dP
        Pm[name] = P[name] - dP
        fp = orc.elastic_step_fwd(st, Pp["lam"], Pp["mu"], Pp["rho"], ax, bx, ay, by, dt, dx,
                                  dy, NX, NY)
        fm = orc.elastic_step_fwd(st, Pm["lam"], Pm["mu"], Pm["rho"], ax, bx, ay, by, dt, dx,
                                  dy, NX, NY)
        fd = np.dot(fp - fm, w) / 2
        assert abs(fd - np.dot(G, dP)) <= 1e-7 * abs(fd), name


def test_elastic_golden_reproduces(orc):
    g = golden("elastic_small.npz")
    NX, NY, T = int(g["NX"]), int(g["NY"]), int(g["NSTEP"])
    ax, bx, kx, ay, by, ky = orc.elastic_cpml(NX, NY, float(g["dx"]), float(g["dy"]),
                                              float(g["dt"]), int(g["npml"]),
                                              float(g["vp_ref"]), float(g["f0"]))
    assert np.allclose(ax, g["ax"], rtol=1e-15, atol=0) and np.allclose(by, g["by"], rtol=1e-15)
    r = orc.elastic_forward(NX, NY, T, float(g["dt"]), float(g["dx"]), float(g["dy"]), ax, bx,
                            ay, by, g["lam"], g["mu"], g["rho"], g["srci"], g["srcj"],
                            g["srctype"], g["srcv"], g["rcvi"], g["rcvj"], g["rcvtype"])
    assert np.linalg.norm(r - g["rcvv"]) <= 1e-14 * np.linalg.norm(g["rcvv"])


def test_elastic_loss_finite_differences(orc):
    g = golden("elastic_small.npz")
    NX, NY, T = int(g["NX"]), int(g["NY"]), 40
    N = (NX + 2) * (NY + 2)
    a = dict(dt=float(g["dt"]), dx=float(g["dx"]), dy=float(g["dy"]))
    obs = g["obs"][:, :T + 1].copy()
    base = [g[k] for k in ("lam", "mu", "rho")]
    def loss(l, m, r):
        return orc.elastic_gradient(NX, NY, T, a["dt"], a["dx"], a["dy"], g["ax"], g["bx"],
                                    g["ay"], g["by"], l, m, r, g["srci"], g["srcj"],
                                    g["srctype"], g["srcv"], g["rcvi"], g["rcvj"],
                                    g["rcvtype"], obs)
    L, gl, gm, gr = loss(*base)
    rng = np.random.default_rng(1)
    for k, G in enumerate((gl, gm, gr)):
        d = rng.standard_normal(N) * base[k] * 1e-4
        p = list(base); p[k] = base[k] + d
        m = list(base); m[k] = base[k] - d
        fd = (loss(*p)[0] - loss(*m)[0]) / 2
        assert abs(fd - np.dot(G, d)) <= 1e-4 * abs(fd), k


def test_acoustic_source_gradient_finite_differences(orc):
    """d loss / d srcv from the oracle's adjoint equals central differences of
    the loss (two sources, one on a receiver's cell); row 0 is never injected."""
    rng = np.random.default_rng(4)
    NX, NY, T = 20, 16, 40
    N = (NX + 2) * (NY + 2)
    dt, h = 1e-3, 10.0
    vp = 2000 + 500 * rng.random(N)
    s, t = orc.acoustic_pml(NX, NY, h, h, 5, 2000.0)
    srci, srcj = [11, 8], [6, 3]
    srcv = rng.standard_normal((T, 2)) * 1e3
    rcvi, rcvj = np.arange(3, 19), np.full(16, 3)
    obs = orc.acoustic_forward(NX, NY, T, dt, h, h, s, t, vp * 1.03, srci, srcj, srcv, rcvi,
                               rcvj)
    _, _, gs = orc.acoustic_gradient(NX, NY, T, dt, h, h, s, t, vp, srci, srcj, srcv, rcvi,
                                     rcvj, obs, want_src=True)
    assert gs.shape == (T, 2) and np.all(gs[0] == 0.0)
    for (row, k) in [(1, 0), (7, 0), (20, 1), (T - 1, 1), (T - 1, 0)]:
        e = 1.0
        sp, sm = srcv.copy(), srcv.copy()
        sp[row, k] += e
        sm[row, k] -= e
        lp = orc.acoustic_gradient(NX, NY, T, dt, h, h, s, t, vp, srci, srcj, sp, rcvi, rcvj,
                                   obs)[0]
        lm = orc.acoustic_gradient(NX, NY, T, dt, h, h, s, t, vp, srci, srcj, sm, rcvi, rcvj,
                                   obs)[0]
        fd = (lp - lm) / (2 * e)
        assert abs(fd - gs[row, k]) <= 1e-7 * max(abs(fd), 1e-12 * abs(lp)), (row, k, fd,
                                                                             gs[row, k])


def test_elastic_source_gradient_finite_differences(orc):
    """d loss / d srcv from the oracle's elastic adjoint equals central
    differences of the loss: one source of each field type (one on a
    receiver's cell, one on the padded ring) and an ignored type."""
    g = golden("elastic_small.npz")
    NX, NY, T = int(g["NX"]), int(g["NY"]), 30
    a = dict(dt=float(g["dt"]), dx=float(g["dx"]), dy=float(g["dy"]))
    rng = np.random.default_rng(6)
    srci = np.array([10, 15, 8, 20, 12, 1, 9])
    srcj = np.array([9, 12, 14, 7, 10, 5, 9])
    srct = np.array([0, 1, 2, 3, 4, 2, 7])
    srcv = rng.standard_normal((T, len(srci))) * 1e2
    rcvi, rcvj, rcvt = g["rcvi"], g["rcvj"], g["rcvtype"]
    srci[0], srcj[0], srct[0] = rcvi[0], rcvj[0], rcvt[0] if rcvt[0] <= 4 else 0
    obs = g["obs"][:, :T + 1].copy()
    lam, mu, rho = g["lam"], g["mu"], g["rho"]

    def run(sv, want=False):
        return orc.elastic_gradient(NX, NY, T, a["dt"], a["dx"], a["dy"], g["ax"], g["bx"],
                                    g["ay"], g["by"], lam, mu, rho, srci, srcj, srct, sv, rcvi,
                                    rcvj, rcvt, obs, want_src=want)

    L, _, _, _, gs = run(srcv, True)
    assert gs.shape == (T, len(srci)) and np.all(gs[:, -1] == 0.0)
    assert L == run(srcv)[0]
    # the loss is quadratic in srcv, so central differences are exact up to
    # rounding of the loss (~1e-16 L / e): a large step keeps that below the
    # stress-source gradients, which are small in these units
    for row, k in [(0, 0), (5, 1), (12, 2), (20, 3), (T - 1, 4), (9, 5), (T - 2, 0)]:
        e = 1e4
        sp, sm = srcv.copy(), srcv.copy()
        sp[row, k] += e
        sm[row, k] -= e
        lp, lm = run(sp)[0], run(sm)[0]
        fd = (lp - lm) / (2 * e)
        tol = 1e-7 * abs(fd) + 1e-15 * max(lp, lm) / e
        assert abs(fd - gs[row, k]) <= tol, (row, k, fd, gs[row, k])
