"""The FP64 plans' specialised PML forms are algebraic rewrites of the general
acoustic update and of its adjoint.

The FP64 step kernels take, per warp, one of three forms instead of the
general one (with its divides): sigma rows only (tau = 0), tau columns only
(sigma = 0), and corners (both), with the damping factors taken from tables:
r = 1 / (1 + s dt/2), ar = (1 - s dt/2) r, e = 1 - s dt, ex = s dt / (2 hx),
ey = s dt / (2 hy) per row (s = sigma) or per column (s = tau), and in the
corners 1/den from a per-cell table with (1 - s dt/2) / (1 + s dt/2) = 2 r - 1.
This restates both the general form (as written in the w-form step of
src/Core.jl:504-549 and its transpose) and the three specialised forms in
numpy on random inputs and checks they agree to FP64 rounding.  The CUDA
kernels themselves are checked against the oracle on the GPU; this pins the
algebra they rely on.  Test infrastructure only."""
import numpy as np
import pytest

DT, HX, HY = 1e-3, 10.0, 12.5
HDT = DT / 2
CX, CY = (DT / HX) ** 2, (DT / HY) ** 2
KXY = 2 * DT * DT / HX / HX + 2 * DT * DT / HY / HY
FX, FY = DT * DT / (2 * HX), DT * DT / (2 * HY)
EX, EY = DT / 2 / HX, DT / 2 / HY
N = 4096


def tables(s):
    """The damping tables of profile values s (KT_R, KT_AR, KT_E, KT_EX, KT_EY)."""
    r = 1.0 / (1.0 + s * HDT)
    return dict(r=r, ar=(1.0 - s * HDT) * r, e=1.0 - s * DT, ex=s * EX, ey=s * EY)


def rng_fields(seed):
    g = np.random.default_rng(seed)
    f = {k: g.standard_normal(N) for k in
         ("w0", "wp", "wm", "wN", "wS", "wo", "p0", "pp", "pm", "q0", "qN", "qS",
          "gu0", "gum", "gu1", "gp0", "gpm", "gp1", "gq", "ln", "ypl", "ymr", "yrl", "yrr")}
    f.update(c0=g.uniform(4e6, 1.2e7, N), cm=g.uniform(4e6, 1.2e7, N), c1=g.uniform(4e6, 1.2e7, N))
    return f, g


def profiles(g, kind):
    """sigma of rows i-1, i, i+1 and tau of the column for a warp kind."""
    sg = [g.uniform(0, 150, N) for _ in range(3)]
    tau = g.uniform(0, 150, N)
    if kind == 1:
        tau = np.zeros(N)
    elif kind == 2:
        sg = [np.zeros(N)] * 3
    return sg, tau


def forward_general(f, sg, tau):
    s = sg + tau
    v = ((2 - sg * tau * DT * DT - KXY * f["c0"]) * f["w0"] + f["c0"] * CX * (f["wp"] + f["wm"])
         + f["c0"] * CY * (f["wN"] + f["wS"]) + FX * (f["pp"] - f["pm"]) + FY * (f["qN"] - f["qS"])
         - (1 - s * HDT) * f["wo"]) / (1 + s * HDT)
    po = (1 - DT * sg) * f["p0"] + EX * f["c0"] * (tau - sg) * (f["wp"] - f["wm"])
    qo = (1 - DT * tau) * f["q0"] + EY * f["c0"] * (sg - tau) * (f["wN"] - f["wS"])
    return v, po, qo


def forward_kind(f, sg, tau, kind):
    c = f["c0"]
    lap = (2 - KXY * c) * f["w0"] + c * CX * (f["wp"] + f["wm"]) + c * CY * (f["wN"] + f["wS"])
    pq = FX * (f["pp"] - f["pm"]) + FY * (f["qN"] - f["qS"])
    if kind in (1, 2):
        t = tables(sg if kind == 1 else tau)
        v = (lap + pq) * t["r"] - t["ar"] * f["wo"]
        if kind == 1:
            po = t["e"] * f["p0"] - t["ex"] * c * (f["wp"] - f["wm"])
            qo = f["q0"] + t["ey"] * c * (f["wN"] - f["wS"])
        else:
            po = f["p0"] + t["ex"] * c * (f["wp"] - f["wm"])
            qo = t["e"] * f["q0"] - t["ey"] * c * (f["wN"] - f["wS"])
        return v, po, qo
    ts = tables(sg)
    rd = 1.0 / (1.0 + (sg + tau) * HDT)
    v = ((2 - sg * tau * DT * DT - KXY * c) * f["w0"] + c * CX * (f["wp"] + f["wm"])
         + c * CY * (f["wN"] + f["wS"]) + pq) * rd - (2 * rd - 1) * f["wo"]
    po = ts["e"] * f["p0"] + c * (EX * tau - ts["ex"]) * (f["wp"] - f["wm"])
    qo = (1 - DT * tau) * f["q0"] + c * (ts["ey"] - EY * tau) * (f["wN"] - f["wS"])
    return v, po, qo


def adjoint_general(f, sg, tau):
    sgm, sg0, sgp = sg
    inv = [1 / (1 + (x + tau) * HDT) for x in sg]
    gui, guim, guip = f["gu0"] * inv[1], f["gum"] * inv[0], f["gu1"] * inv[2]
    by = f["c0"] * CY * gui
    eyg = EY * f["c0"] * (sg0 - tau) * f["gq"]
    XPm = f["cm"] * CX * guim + EX * f["cm"] * (tau - sgm) * f["gpm"]
    XMp = f["c1"] * CX * guip - EX * f["c1"] * (tau - sgp) * f["gp1"]
    s = sg0 + tau
    nu = (-(1 - s * HDT) * inv[1] * f["ln"] + (2 - sg0 * tau * DT * DT - KXY * f["c0"]) * gui
          + XPm + XMp + f["ypl"] + f["ymr"])
    np_ = (1 - DT * sg0) * f["gp0"] + FX * guim - FX * guip
    nq = (1 - DT * tau) * f["gq"] + f["yrl"] - f["yrr"]
    dx, dy = f["wp"] - f["wm"], f["wN"] - f["wS"]
    g = ((-KXY * f["w0"] + CX * (f["wp"] + f["wm"]) + CY * (f["wN"] + f["wS"])) * gui
         + EX * (tau - sg0) * dx * f["gp0"] + EY * (sg0 - tau) * dy * f["gq"])
    return nu, np_, nq, g, by + eyg, by - eyg, FY * gui


def adjoint_kind(f, sg, tau, kind):
    sgm, sg0, sgp = sg
    c0, cm, c1 = f["c0"], f["cm"], f["c1"]
    dx, dy = f["wp"] - f["wm"], f["wN"] - f["wS"]
    lapw = -KXY * f["w0"] + CX * (f["wp"] + f["wm"]) + CY * (f["wN"] + f["wS"])
    if kind == 1:
        tm, t0, tp = (tables(x) for x in sg)
        gui, guim, guip = f["gu0"] * t0["r"], f["gum"] * tm["r"], f["gu1"] * tp["r"]
        ey = t0["ey"]
        XPm = cm * (CX * guim - tm["ex"] * f["gpm"])
        XMp = c1 * (CX * guip + tp["ex"] * f["gp1"])
        nu = -t0["ar"] * f["ln"] + (2 - KXY * c0) * gui + XPm + XMp + f["ypl"] + f["ymr"]
        np_ = t0["e"] * f["gp0"] + FX * (guim - guip)
        nq = f["gq"] + f["yrl"] - f["yrr"]
        g = lapw * gui - t0["ex"] * dx * f["gp0"] + t0["ey"] * dy * f["gq"]
    elif kind == 2:
        t = tables(tau)
        gui, guim, guip = f["gu0"] * t["r"], f["gum"] * t["r"], f["gu1"] * t["r"]
        ey = -t["ey"]
        XPm = cm * (CX * guim + t["ex"] * f["gpm"])
        XMp = c1 * (CX * guip - t["ex"] * f["gp1"])
        nu = -t["ar"] * f["ln"] + (2 - KXY * c0) * gui + XPm + XMp + f["ypl"] + f["ymr"]
        np_ = f["gp0"] + FX * (guim - guip)
        nq = t["e"] * f["gq"] + f["yrl"] - f["yrr"]
        g = lapw * gui + t["ex"] * dx * f["gp0"] - t["ey"] * dy * f["gq"]
    else:
        tm, t0, tp = (tables(x) for x in sg)
        rd = [1 / (1 + (x + tau) * HDT) for x in sg]
        gui, guim, guip = f["gu0"] * rd[1], f["gum"] * rd[0], f["gu1"] * rd[2]
        ey = t0["ey"] - EY * tau
        XPm = cm * (CX * guim + (EX * tau - tm["ex"]) * f["gpm"])
        XMp = c1 * (CX * guip - (EX * tau - tp["ex"]) * f["gp1"])
        nu = (-(2 * rd[1] - 1) * f["ln"] + (2 - sg0 * tau * DT * DT - KXY * c0) * gui
              + XPm + XMp + f["ypl"] + f["ymr"])
        np_ = t0["e"] * f["gp0"] + FX * (guim - guip)
        nq = (1 - DT * tau) * f["gq"] + f["yrl"] - f["yrr"]
        g = lapw * gui + (EX * tau - t0["ex"]) * dx * f["gp0"] + (t0["ey"] - EY * tau) * dy * f["gq"]
    by = c0 * CY * gui
    eyg = ey * c0 * f["gq"]
    return nu, np_, nq, g, by + eyg, by - eyg, FY * gui


def close(a, b):
    return np.max(np.abs(a - b)) <= 1e-13 * max(np.max(np.abs(b)), 1e-300)


@pytest.mark.parametrize("kind", [1, 2, 3])
def test_forward_kinds_are_rewrites_of_the_general_update(kind):
    f, g = rng_fields(kind)
    sg, tau = profiles(g, kind)
    for a, b in zip(forward_kind(f, sg[1], tau, kind), forward_general(f, sg[1], tau)):
        assert close(a, b)


@pytest.mark.parametrize("kind", [1, 2, 3])
def test_adjoint_kinds_are_rewrites_of_the_general_transpose(kind):
    f, g = rng_fields(10 + kind)
    sg, tau = profiles(g, kind)
    for a, b in zip(adjoint_kind(f, sg, tau, kind), adjoint_general(f, sg, tau)):
        assert close(a, b)


def test_corner_identity():
    """(1 - s dt/2) / (1 + s dt/2) = 2 / (1 + s dt/2) - 1, the corners' 2 r - 1."""
    s = np.random.default_rng(0).uniform(0, 500, N)
    r = 1 / (1 + s * HDT)
    assert np.max(np.abs((1 - s * HDT) * r - (2 * r - 1))) <= 4e-16
