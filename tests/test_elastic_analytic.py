"""Analytic pins of the elastic step (src/Core.jl:96-228), independent of the
oracle's code: exact discrete plane waves and known-answer steps.

Staggering, read off the four derivative stencils (positions in cells):
vx at (i, j), vy at (i+1/2, j+1/2), sigma_xx / sigma_yy at (i+1/2, j),
sigma_xy at (i, j+1/2).  The staggered fourth-order derivative
(27 (a_0 - a_-1) - (a_1 - a_-2)) / (24 h) maps exp(i k x) to
i K exp(i k x) with K = (27 sin(k h / 2) - sin(3 k h / 2)) / (12 h).

A plane P-wave along x in a homogeneous medium with the CPML off (a = 0, so
the memory variables stay 0) has vx = v_n exp(i k x), sigma_xx = s_n exp(i k
(x + h/2)), sigma_yy = (lambda / (lambda + 2 mu)) sigma_xx, vy = sigma_xy = 0.
One step (fw1 updates the stresses from the old velocities, fw3 the
velocities from the new stresses) is the 2 x 2 map

    s_{n+1} = s_n + i dt (lambda + 2 mu) K v_n
    v_{n+1} = v_n + i (dt / rho) K s_{n+1},

with determinant 1 and trace 2 - (vp dt K)^2, so its eigenvalues are
exp(+-i w dt) with the discrete dispersion relation

    sin(w dt / 2) = vp dt (27 sin(k h / 2) - sin(3 k h / 2)) / (24 h).

The same holds for an S-wave (vs = sqrt(mu / rho); vy and sigma_xy, fw2 / fw4)
and for propagation along y.  Cells farther than 4 n + 4 cells from the
grid's edge (the update boxes end there, and a step moves information at
most 4 cells) carry the plane wave exactly after n steps; the tests compare
them with the 2 x 2 map to 1e-12 of the wave's amplitude, on the oracle (CPU)
and through ads_elastic_step_fwd_f64 (GPU).

Material averages (fw1: lambda, mu over (i, j), (i+1, j); fw2: mu over
(i, j), (i, j+1); fw3: rho at (i, j); fw4: rho over the four cells around
(i+1/2, j+1/2)) are pinned by single steps from fields that are linear in x
or y, whose staggered derivative is exactly 1: in a random medium one step
then writes dt times the averaged material (or dt over the averaged density).
"""
import numpy as np
import pytest

NF = 13
VX, VY, SXX, SYY, SXY = range(5)
TOL = 1e-12


def K_of(k, h):
    return (27 * np.sin(k * h / 2) - np.sin(3 * k * h / 2)) / (12 * h)


def plane_wave(mode, axis, NX, NY, hx, hy, k, lam, mu, rho, dt, n, K=None):
    """(state_0, state_n) of the exact discrete plane wave after n steps, and the
    mask of cells to compare; K replaces the stencil's symbol K_of."""
    h = hx if axis == "x" else hy
    KK = (K or K_of)(k, h)
    if mode == "P":
        Mmod = lam + 2 * mu
        ratio = lam / (lam + 2 * mu)
    else:
        Mmod = mu
        ratio = 0.0
    a = 1j * dt * Mmod * KK
    b = 1j * dt / rho * KK
    M = np.array([[1, a], [b, 1 + a * b]], dtype=complex)
    w = np.arccos(np.trace(M).real / 2) / dt
    # check the closed-form dispersion relation against the map itself
    assert abs(np.sin(w * dt / 2) - np.sqrt(Mmod / rho) * dt * KK / 2) < 1e-14
    s0, v0 = 0.7 + 0.2j, -0.3 + 0.5j
    Mn = np.linalg.matrix_power(M, n)
    sn, vn = Mn @ np.array([s0, v0])
    I = np.arange(NX + 2, dtype=np.float64)[:, None] * hx
    J = np.arange(NY + 2, dtype=np.float64)[None, :] * hy
    pos = {  # (x, y) of each field's samples
        VX: (I, J), VY: (I + hx / 2, J + hy / 2), SXX: (I + hx / 2, J), SYY: (I + hx / 2, J),
        SXY: (I, J + hy / 2)}
    if mode == "P" and axis == "x":
        vel, fields = VX, ((SXX, 1.0), (SYY, ratio))
    elif mode == "P":
        vel, fields = VY, ((SYY, 1.0), (SXX, ratio))
    elif axis == "x":
        vel, fields = VY, ((SXY, 1.0),)
    else:
        vel, fields = VX, ((SXY, 1.0),)

    def fill(s, v):
        st = np.zeros((NF, NX + 2, NY + 2))
        x, y = pos[vel]
        ph = np.exp(1j * k * (x if axis == "x" else y))
        st[vel] = np.broadcast_to((v * ph).real, (NX + 2, NY + 2))
        for f, r in fields:
            x, y = pos[f]
            ph = np.exp(1j * k * (x if axis == "x" else y))
            st[f] = np.broadcast_to((r * s * ph).real, (NX + 2, NY + 2))
        return st

    m = 4 * n + 4
    mask = np.zeros((NX + 2, NY + 2), dtype=bool)
    mask[m:NX + 2 - m, m:NY + 2 - m] = True
    amp = max(abs(s0), abs(v0), abs(sn), abs(vn))
    return fill(s0, v0), fill(sn, vn), mask, amp


def no_cpml(orc, NX, NY, hx, hy, dt):
    """CPML profiles with every side off: a = 0, so the memory variables stay 0."""
    ax, bx, kx, ay, by, ky = orc.elastic_cpml(NX, NY, hx, hy, dt, 10, 3000.0, 10.0, use_pml=0)
    assert not ax.any() and not ay.any()
    return ax, bx, ay, by


CASES = [("P", "x"), ("P", "y"), ("S", "x"), ("S", "y")]


def _setup(mode, axis, n, K=None):
    NX, NY, hx, hy = 200, 180, 10.0, 12.5
    lam, mu, rho = 9.1e9, 5.2e9, 2300.0
    vp = np.sqrt((lam + 2 * mu) / rho)
    dt = 0.35 * min(hx, hy) / vp
    h = hx if axis == "x" else hy
    k = 2 * np.pi / (7.3 * h)  # about 7 cells per wavelength: far from the continuum limit
    st0, stn, mask, amp = plane_wave(mode, axis, NX, NY, hx, hy, k, lam, mu, rho, dt, n, K)
    N = (NX + 2) * (NY + 2)
    mats = [np.full(N, lam), np.full(N, mu), np.full(N, rho)]
    return NX, NY, hx, hy, dt, mats, st0, stn, mask, amp


def _check(got, stn, mask, amp):
    got = got.reshape(NF, *mask.shape)
    err = max(np.abs(got[f][mask] - stn[f][mask]).max() for f in range(NF))
    assert err <= TOL * amp, err
    return err


N_STEPS = 16


def _run_oracle(orc, mode, axis, n):
    NX, NY, hx, hy, dt, (lam, mu, rho), st0, stn, mask, amp = _setup(mode, axis, n)
    ax, bx, ay, by = no_cpml(orc, NX, NY, hx, hy, dt)
    st = st0.reshape(-1)
    for _ in range(n):
        st = orc.elastic_step_fwd(st, lam, mu, rho, ax, bx, ay, by, dt, hx, hy, NX, NY)
    return st, stn, mask, amp


@pytest.mark.parametrize("mode,axis", CASES)
def test_plane_wave_is_an_exact_eigenmode_oracle(orc, mode, axis):
    st, stn, mask, amp = _run_oracle(orc, mode, axis, N_STEPS)
    assert mask.sum() > 2000
    _check(st, stn, mask, amp)


@pytest.mark.parametrize("mode,axis", CASES)
def test_second_order_stencil_would_fail_the_pin(orc, mode, axis):
    """The pin discriminates the stencil: the same wave predicted with the
    second-order symbol K = 2 sin(k h / 2) / h misses the step's result by more
    than 1e-3 of the amplitude, 1e9 times the tolerance."""
    st, _, mask, amp = _run_oracle(orc, mode, axis, N_STEPS)
    stn2 = _setup(mode, axis, N_STEPS, K=lambda k, h: 2 * np.sin(k * h / 2) / h)[7]
    got = st.reshape(NF, *mask.shape)
    err = max(np.abs(got[f][mask] - stn2[f][mask]).max() for f in range(NF))
    assert err > 1e-3 * amp


@pytest.mark.gpu
@pytest.mark.parametrize("mode,axis", CASES)
def test_plane_wave_is_an_exact_eigenmode_gpu(ads, orc, cuda, mode, axis):
    import torch

    n = N_STEPS
    NX, NY, hx, hy, dt, (lam, mu, rho), st0, stn, mask, amp = _setup(mode, axis, n)
    ax, bx, ay, by = no_cpml(orc, NX, NY, hx, hy, dt)
    p = ads.ElasticPropagatorParams(NX=NX, NY=NY, DELTAX=hx, DELTAY=hy, DELTAT=dt)
    T = lambda a: torch.as_tensor(np.ascontiguousarray(a), dtype=torch.float64, device=cuda)
    prof = (T(ax), T(bx), T(np.ones_like(ax)), T(ay), T(by), T(np.ones_like(ay)))
    st = T(st0.reshape(NF, -1))
    for _ in range(n):
        st = ads.elastic_one_step(p, T(rho), T(lam), T(mu), st, prof)
    _check(st.cpu().numpy(), stn, mask, amp)


# ------------------------------------------------------------ material averages

def _linear_step(step, field, along, seed=3):
    """One step from a state whose only non-zero field is `field`, linear in x or y
    (value = position in metres, so its staggered derivative is exactly 1)."""
    NX, NY, hx, hy, dt = 20, 18, 10.0, 12.5, 1e-3
    rng = np.random.default_rng(seed)
    shape = (NX + 2, NY + 2)
    lam = 6e9 * (1 + rng.random(shape))
    mu = 3e9 * (1 + rng.random(shape))
    rho = 2000.0 * (1 + rng.random(shape))
    I = np.arange(NX + 2, dtype=np.float64)[:, None] * hx
    J = np.arange(NY + 2, dtype=np.float64)[None, :] * hy
    off = {VX: (0, 0), VY: (0.5, 0.5), SXX: (0.5, 0), SYY: (0.5, 0), SXY: (0, 0.5)}[field]
    st = np.zeros((NF,) + shape)
    st[field] = np.broadcast_to(I + off[0] * hx if along == "x" else J + off[1] * hy, shape)
    out = step(st.reshape(-1), lam, mu, rho, dt, hx, hy, NX, NY).reshape((NF,) + shape)
    return out, st, lam, mu, rho, dt, NX, NY


def _oracle_step(orc):
    def step(st, lam, mu, rho, dt, hx, hy, NX, NY):
        ax, bx, ay, by = no_cpml(orc, NX, NY, hx, hy, dt)
        return orc.elastic_step_fwd(st, lam.reshape(-1), mu.reshape(-1), rho.reshape(-1), ax,
                                    bx, ay, by, dt, hx, hy, NX, NY)
    return step


def _gpu_step(ads, orc, cuda):
    import torch

    def step(st, lam, mu, rho, dt, hx, hy, NX, NY):
        ax, bx, ay, by = no_cpml(orc, NX, NY, hx, hy, dt)
        p = ads.ElasticPropagatorParams(NX=NX, NY=NY, DELTAX=hx, DELTAY=hy, DELTAT=dt)
        T = lambda a: torch.as_tensor(np.ascontiguousarray(a).reshape(-1), dtype=torch.float64,
                                      device=cuda)
        prof = (T(ax), T(bx), T(np.ones_like(ax)), T(ay), T(by), T(np.ones_like(ay)))
        return ads.elastic_one_step(p, T(rho), T(lam), T(mu), T(st).reshape(NF, -1),
                                    prof).cpu().numpy()
    return step


def _averages_hold(step):
    # vx = x: dvx/dx = 1 at the stress points (i+1/2, j), box i in 2:NX, j in 3:NY+1
    out, st, lam, mu, rho, dt, NX, NY = _linear_step(step, VX, "x")
    lam_ = 0.5 * (lam[1:NX, 2:NY + 1] + lam[2:NX + 1, 2:NY + 1])
    mu_ = 0.5 * (mu[1:NX, 2:NY + 1] + mu[2:NX + 1, 2:NY + 1])
    np.testing.assert_allclose(out[SXX, 1:NX, 2:NY + 1], dt * (lam_ + 2 * mu_), rtol=1e-14)
    np.testing.assert_allclose(out[SYY, 1:NX, 2:NY + 1], dt * lam_, rtol=1e-14)
    # vy = x: dvy/dx = 1 at the shear points (i, j+1/2), box i in 3:NX+1, j in 2:NY
    out, st, lam, mu, rho, dt, NX, NY = _linear_step(step, VY, "x")
    mu_xy = 0.5 * (mu[2:NX + 1, 1:NY] + mu[2:NX + 1, 2:NY + 1])
    np.testing.assert_allclose(out[SXY, 2:NX + 1, 1:NY], dt * mu_xy, rtol=1e-14)
    # sigma_xx = x: d/dx = 1 at vx points (i, j), box i in 3:NX+1, j in 3:NY+1
    out, st, lam, mu, rho, dt, NX, NY = _linear_step(step, SXX, "x")
    np.testing.assert_allclose(out[VX, 2:NX + 1, 2:NY + 1], dt / rho[2:NX + 1, 2:NY + 1],
                               rtol=1e-14)
    # sigma_yy = y: d/dy = 1 at vy points (i+1/2, j+1/2), box i in 2:NX, j in 2:NY
    out, st, lam, mu, rho, dt, NX, NY = _linear_step(step, SYY, "y")
    rho4 = 0.25 * (rho[1:NX, 1:NY] + rho[2:NX + 1, 1:NY] + rho[2:NX + 1, 2:NY + 1] +
                   rho[1:NX, 2:NY + 1])
    np.testing.assert_allclose(out[VY, 1:NX, 1:NY], dt / rho4, rtol=1e-14)


def test_material_averages_oracle(orc):
    _averages_hold(_oracle_step(orc))


@pytest.mark.gpu
def test_material_averages_gpu(ads, orc, cuda):
    _averages_hold(_gpu_step(ads, orc, cuda))
