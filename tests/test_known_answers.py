"""Known-answer tests that pin the oracle's step coefficients and time-index
conventions with values written out by hand (no reference run involved):

- the acoustic step (AcousticOneStepCpu.h:1-48 / src/Core.jl:504-549) applied
  to a unit impulse in a PML-free medium;
- the acoustic loop (src/Core.jl:562-620): slots 0 and 1 are zero, slot
  k >= 2 is the step of slots k-1, k-2 plus srcv[k-1] dt^2 at the source, so
  srcv row 0 is never injected;
- the elastic loop (src/Core.jl:31-94): slot 0 is zero, slot n >= 1 is the
  step of slot n-1 plus srcv[n-1] (AddSource, no dt factor).

Every GPU path is checked against this oracle, so these conventions carry
over to it.  Test infrastructure only."""
import numpy as np
import pytest


def test_acoustic_impulse_step(orc):
    NX, NY, dt, hx, hy, cv = 9, 7, 1e-3, 10.0, 8.0, 2500.0 ** 2
    shape = (NX + 2, NY + 2)
    w = np.zeros(shape)
    w[5, 4] = 1.0
    z = np.zeros(shape).reshape(-1)
    c = np.full(shape, cv).reshape(-1)
    for variant in (0, 1):
        u, p, q = (np.asarray(a).reshape(shape) for a in orc.acoustic_step_fwd(
            w.reshape(-1), z, z, z, z, z, c, dt, hx, hy, NX, NY, variant=variant))
        want = np.zeros(shape)
        want[5, 4] = 2 - 2 * dt ** 2 / hx ** 2 * cv - 2 * dt ** 2 / hy ** 2 * cv
        want[4, 4] = want[6, 4] = cv * (dt / hx) ** 2
        want[5, 3] = want[5, 5] = cv * (dt / hy) ** 2
        assert np.abs(u - want).max() <= 1e-15 * abs(want[5, 4]), variant
        assert not p.any() and not q.any()  # sigma = tau = 0: no PML auxiliaries


def test_acoustic_source_and_receiver_time_convention(orc):
    """One source and receivers on it and on a neighbour in a constant, PML-free
    medium: the first three slots by hand."""
    NX, NY, T, dt, h, cv = 11, 9, 4, 1e-3, 10.0, 2000.0 ** 2
    N = (NX + 2) * (NY + 2)
    z = np.zeros(N)
    vp = np.full(N, np.sqrt(cv))
    a = np.array([[7.0], [3.0], [-2.0], [5.0]])
    si, sj = [6], [5]
    rcvi, rcvj = np.array([6, 7, 6]), np.array([5, 5, 6])
    tr = orc.acoustic_forward(NX, NY, T, dt, h, h, z, z, vp, si, sj, a, rcvi, rcvj)
    d2 = dt * dt
    centre = 2 - 2 * d2 / h ** 2 * cv - 2 * d2 / h ** 2 * cv
    assert tr.shape == (T + 1, 3)
    assert np.all(tr[0] == 0) and np.all(tr[1] == 0)  # slots 0, 1; row 0 unused
    assert tr[2, 0] == pytest.approx(a[1, 0] * d2, rel=1e-15) and tr[2, 1] == tr[2, 2] == 0
    assert tr[3, 0] == pytest.approx(centre * a[1, 0] * d2 + a[2, 0] * d2, rel=1e-13)
    assert tr[3, 1] == pytest.approx(cv * d2 / h ** 2 * a[1, 0] * d2, rel=1e-13)
    assert tr[3, 2] == pytest.approx(cv * d2 / h ** 2 * a[1, 0] * d2, rel=1e-13)


def test_elastic_source_time_convention(orc):
    """A vx source a with a vx receiver on its cell, in a homogeneous medium
    without CPML (a = 0, b = 1): slot 1 holds a[0] exactly (the step of the
    zero state is zero); slot 2 holds a[0] + a[1] plus one step of the
    impulse, by hand: fw1 / fw2 turn it into stresses lambda+2mu, lambda, mu
    times dt (27, -27, -1, 1) a[0] / (24 h) around it, and fw3 brings them
    back to vx(s) with weight (-27 * 27 - 27 * 27 - 1 - 1) / (24 h)^2 per
    direction, i.e. vx_2(s) = a[0] + a[1] - 1460 a[0] dt^2 ((lambda + 2 mu) /
    dx^2 + mu / dy^2) / (576 rho)."""
    NX, NY, T, dt, dx, dy = 12, 10, 3, 1e-4, 10.0, 8.0
    N = (NX + 2) * (NY + 2)
    L, M, R = 2e10, 1e10, 2500.0
    a = np.array([[4.0], [1.5], [0.5]])
    tr = orc.elastic_forward(NX, NY, T, dt, dx, dy, np.zeros(2 * NX), np.ones(2 * NX),
                             np.zeros(2 * NY), np.ones(2 * NY), np.full(N, L), np.full(N, M),
                             np.full(N, R), [7], [6], [0], a, [7], [6], [0])
    assert tr.shape == (1, T + 1)
    assert tr[0, 0] == 0 and tr[0, 1] == a[0, 0]
    want = a[0, 0] + a[1, 0] - 1460 * a[0, 0] * dt ** 2 * ((L + 2 * M) / dx ** 2 +
                                                          M / dy ** 2) / (576 * R)
    assert tr[0, 2] == pytest.approx(want, rel=1e-13)
    assert abs(tr[0, 2] - (a[0, 0] + a[1, 0])) > 1e-3  # the step's share is not negligible
