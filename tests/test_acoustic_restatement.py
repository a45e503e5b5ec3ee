"""A second, independent restatement of the reference's TF-composed acoustic
steps, written with numpy slices straight from src/Core.jl:504-549:
one_step (PropagatorKernel 0, phi / psi from the new u) and
acoustic_one_step_customop_ref (PropagatorKernel 2, phi / psi from the old
w), with scatter_nd_ops leaving the padded frame at zero.  The u form has no
compiled reference; this checks the C oracle's step and loop in that form
against a restatement that shares no code with it.  The w form is pinned bit
for bit against the compiled AcousticOneStepCpu elsewhere; here it only
checks that the TF composition agrees with it to rounding.  Test
infrastructure only."""
import numpy as np
import pytest


def _step(w, wold, phi, psi, sig, tau, c, dt, hx, hy, NX, NY, new_u):
    """(u, phi, psi) on (NX+2, NY+2) arrays; interior IJ = 2:NX+1 x 2:NY+1."""
    I, Ip, In = slice(1, NX + 1), slice(2, NX + 2), slice(0, NX)
    J, Jp, Jn = slice(1, NY + 1), slice(2, NY + 2), slice(0, NY)
    s, t, cc = sig[I, J], tau[I, J], c[I, J]
    u_in = ((2 - s * t * dt ** 2 - 2 * dt ** 2 / hx ** 2 * cc - 2 * dt ** 2 / hy ** 2 * cc)
            * w[I, J] + cc * (dt / hx) ** 2 * (w[Ip, J] + w[In, J])
            + cc * (dt / hy) ** 2 * (w[I, Jp] + w[I, Jn])
            + (dt ** 2 / (2 * hx)) * (phi[Ip, J] - phi[In, J])
            + (dt ** 2 / (2 * hy)) * (psi[I, Jp] - psi[I, Jn])
            - (1 - (s + t) * dt / 2) * wold[I, J])
    u_in = u_in / (1 + (s + t) / 2 * dt)
    u = np.zeros_like(w)
    u[I, J] = u_in
    f = u if new_u else w
    p = np.zeros_like(w)
    q = np.zeros_like(w)
    p[I, J] = (1.0 - dt * s) * phi[I, J] + dt * cc * (t - s) / (2 * hx) * (f[Ip, J] - f[In, J])
    q[I, J] = (1.0 - dt * t) * psi[I, J] + dt * cc * (s - t) / (2 * hy) * (f[I, Jp] - f[I, Jn])
    return u, p, q


@pytest.mark.parametrize("variant,bitwise", [(1, True), (0, False)])
def test_step_matches_the_oracle(orc, variant, bitwise):
    NX, NY = 17, 13
    shape = (NX + 2, NY + 2)
    rng = np.random.default_rng(7 + variant)
    w, wold, phi, psi = (rng.standard_normal(shape) for _ in range(4))
    sig, tau = rng.random(shape) * 30, rng.random(shape) * 30
    c = (2000 + 500 * rng.random(shape)) ** 2
    dt, hx, hy = 1e-3, 10.0, 12.0
    want = _step(w, wold, phi, psi, sig, tau, c, dt, hx, hy, NX, NY, new_u=variant == 1)
    got = orc.acoustic_step_fwd(*(a.reshape(-1) for a in (w, wold, phi, psi, sig, tau, c)),
                                dt, hx, hy, NX, NY, variant=variant)
    for g, x in zip(got, want):
        g = np.asarray(g).reshape(shape)
        if bitwise:
            assert np.array_equal(g, x)
        else:
            assert np.abs(g - x).max() <= 1e-14 * np.abs(x).max()


def test_u_form_loop_matches_the_oracle(orc):
    """The loop of src/Core.jl:562-620 in the u form (slots 0 and 1 zero; slot
    k = one_step of slots k-1, k-2, then + srcv[k-1] dt^2 at the source) over a
    PML model: the whole history against the oracle's."""
    rng = np.random.default_rng(3)
    NX, NY, T, h, dt = 24, 20, 60, 10.0, 1e-3
    shape = (NX + 2, NY + 2)
    s, t = orc.acoustic_pml(NX, NY, h, h, 6, 2000.0)
    vp = 2000 + 400 * rng.random(shape)
    srci, srcj = np.array([12, 7]), np.array([9, 15])
    srcv = rng.standard_normal((T, 2)) * 1e3
    rcvi, rcvj = np.arange(3, 23), np.full(20, 4)
    sig, tau, c = s.reshape(shape), t.reshape(shape), vp * vp
    U = [np.zeros(shape), np.zeros(shape)]
    phi, psi = np.zeros(shape), np.zeros(shape)
    for k in range(2, T + 1):
        u, phi, psi = _step(U[k - 1], U[k - 2], phi, psi, sig, tau, c, dt, h, h, NX, NY,
                            new_u=True)
        for i, j, v in zip(srci, srcj, srcv[k - 1]):
            u[i - 1, j - 1] += v * dt ** 2
        U.append(u)
    U = np.stack(U)
    _, hist = orc.acoustic_forward(NX, NY, T, dt, h, h, s, t, vp.reshape(-1), srci, srcj,
                                   srcv, rcvi, rcvj, variant=1, keep_history=True)
    assert np.array_equal(hist, U)
