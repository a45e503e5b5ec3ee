"""CPU oracle for ADSeismic's time-stepping hot path -- TEST INFRASTRUCTURE ONLY.

The checker, never the product: only ``tests/``, ``__graft_entry__.smoke()``
and ``bench.py``'s CPU-baseline / reference legs import this module.

Two libraries sit behind it:

* ``_build/liboracle.so`` -- ``oracle.c``, a plain-C restatement of the
  reference's acoustic operator (deps/CustomOps/AcousticOneStepCpu/
  AcousticOneStepCpu.h), its Julia time loops (src/Core.jl), PML/CPML setup,
  the elastic composition (src/Core.jl:96-228) and its hand-derived adjoint.
  Builds anywhere (``make -C oracle``).
* ``_ref/libadsref.so`` -- the reference's OWN CPU operators compiled from the
  reference checkout named by the environment variable ``ADS_REFERENCE_SRC``
  (``make -C oracle ref``); only where that variable names a checkout.  Used
  to pin the restatement.

All arrays are float64 numpy, flat row-major (NX+2)x(NY+2) with j contiguous;
source/receiver indices are 1-based into the padded grid (reference convention).
"""
from __future__ import annotations

import ctypes as C
import os
import subprocess

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(HERE, "_build", "liboracle.so")
REF_PATH = os.path.join(HERE, "_ref", "libadsref.so")

_dp = C.POINTER(C.c_double)
_ip = C.POINTER(C.c_int64)


def reference_checkout():
    """The reference checkout named by ADS_REFERENCE_SRC, or None."""
    src = os.environ.get("ADS_REFERENCE_SRC", "")
    return src if src and os.path.isdir(src) else None


def build(ref: bool = True) -> None:
    """Compile the restatement and, when ADS_REFERENCE_SRC names a reference
    checkout, _ref."""
    subprocess.run(["make", "-s", "-C", HERE, "all"], check=True)
    src = reference_checkout()
    if ref and src:
        subprocess.run(["make", "-s", "-C", HERE, "ref", "REF=" + src], check=True)


_lib = None
_ref = None


def lib():
    global _lib
    if _lib is None:
        if not os.path.exists(LIB_PATH):
            build(ref=False)
        _lib = C.CDLL(LIB_PATH)
    return _lib


def ref_available() -> bool:
    return os.path.exists(REF_PATH)


def ref():
    global _ref
    if _ref is None:
        _ref = C.CDLL(REF_PATH)
    return _ref


def _d(a):
    return a.ctypes.data_as(_dp) if a is not None else None


def _i(a):
    return a.ctypes.data_as(_ip) if a is not None else None


def _f64(a):
    return np.ascontiguousarray(a, dtype=np.float64)


def _i64(a):
    return np.ascontiguousarray(a, dtype=np.int64)


# ---------------------------------------------------------------- acoustic

def acoustic_step_fwd(w, wold, phi, psi, sigma, tau, c, dt, hx, hy, NX, NY,
                      variant=0, use_ref=False):
    N = (NX + 2) * (NY + 2)
    u, po, qo = np.empty(N), np.empty(N), np.empty(N)
    keep = [_f64(x) for x in (w, wold, phi, psi, sigma, tau, c)]
    args = [_d(x) for x in keep]
    if use_ref:
        assert variant == 0
        ref().ref_acoustic_step_fwd(*args, C.c_double(dt), C.c_double(hx), C.c_double(hy),
                                    C.c_int64(NX), C.c_int64(NY), _d(u), _d(po), _d(qo))
    else:
        lib().orc_acoustic_step_fwd(*args, C.c_double(dt), C.c_double(hx), C.c_double(hy),
                                    C.c_int64(NX), C.c_int64(NY), _d(u), _d(po), _d(qo),
                                    C.c_int(variant))
    return u, po, qo


def acoustic_step_bwd(gu, gphi, gpsi, w, wold, phi, psi, sigma, tau, c, dt, hx, hy,
                      NX, NY, u, phiout, psiout, variant=0, use_ref=False):
    N = (NX + 2) * (NY + 2)
    outs = [np.empty(N) for _ in range(5)]
    keep = [_f64(x) for x in (gu, gphi, gpsi, w, wold, phi, psi, sigma, tau, c)]
    tail = [_f64(x) for x in (u, phiout, psiout)]
    a = [_d(x) for x in outs] + [_d(x) for x in keep] + [
        C.c_double(dt), C.c_double(hx), C.c_double(hy), C.c_int64(NX), C.c_int64(NY)
    ] + [_d(x) for x in tail]
    if use_ref:
        assert variant == 0
        ref().ref_acoustic_step_bwd(*a)
    else:
        lib().orc_acoustic_step_bwd(*a, C.c_int(variant))
    return tuple(outs)  # grad_w, grad_wold, grad_phi, grad_psi, grad_c


def acoustic_pml(NX, NY, hx, hy, npml, vp_ref, Rcoef=0.001, use_pml=15):
    N = (NX + 2) * (NY + 2)
    s, t = np.empty(N), np.empty(N)
    lib().orc_acoustic_pml(C.c_int64(NX), C.c_int64(NY), C.c_double(hx), C.c_double(hy),
                           C.c_int64(npml), C.c_double(vp_ref), C.c_double(Rcoef),
                           C.c_int(use_pml), _d(s), _d(t))
    return s, t


def acoustic_forward(NX, NY, NSTEP, dt, hx, hy, sigma, tau, vp, srci, srcj, srcv,
                     rcvi, rcvj, variant=0, keep_history=False, use_ref=False):
    N = (NX + 2) * (NY + 2)
    srci, srcj, rcvi, rcvj = map(_i64, (srci, srcj, rcvi, rcvj))
    srcv = _f64(srcv).reshape(-1)
    sigma, tau, vp = map(_f64, (sigma, tau, vp))
    nsrc, nrcv = len(srci), len(rcvi)
    assert srcv.size >= NSTEP * nsrc
    rcvv = np.zeros((NSTEP + 1) * nrcv)
    hist = np.empty((NSTEP + 1) * N) if keep_history else None
    if use_ref:
        assert variant == 0 and not keep_history
        ref().ref_acoustic_forward(C.c_int64(NX), C.c_int64(NY), C.c_int64(NSTEP),
                                   C.c_double(dt), C.c_double(hx), C.c_double(hy),
                                   _d(sigma), _d(tau), _d(vp), C.c_int64(nsrc), _i(srci),
                                   _i(srcj), _d(srcv), C.c_int64(nrcv), _i(rcvi), _i(rcvj),
                                   _d(rcvv))
    else:
        lib().orc_acoustic_forward(C.c_int64(NX), C.c_int64(NY), C.c_int64(NSTEP),
                                   C.c_double(dt), C.c_double(hx), C.c_double(hy),
                                   _d(sigma), _d(tau), _d(vp), C.c_int64(nsrc), _i(srci),
                                   _i(srcj), _d(srcv), C.c_int64(nrcv), _i(rcvi), _i(rcvj),
                                   _d(rcvv), _d(hist), C.c_int(variant))
    rcvv = rcvv.reshape(NSTEP + 1, nrcv)
    if keep_history:
        return rcvv, hist.reshape(NSTEP + 1, NX + 2, NY + 2)
    return rcvv


def acoustic_gradient(NX, NY, NSTEP, dt, hx, hy, sigma, tau, vp, srci, srcj, srcv,
                      rcvi, rcvj, obs, variant=0, use_ref=False, want_src=False):
    """(loss, grad_vp), or (loss, grad_vp, grad_srcv (NSTEP, nsrc)) with want_src."""
    N = (NX + 2) * (NY + 2)
    srci, srcj, rcvi, rcvj = map(_i64, (srci, srcj, rcvi, rcvj))
    srcv, obs = _f64(srcv).reshape(-1), _f64(obs).reshape(-1)
    sigma, tau, vp = map(_f64, (sigma, tau, vp))
    g = np.empty(N)
    args = [C.c_int64(NX), C.c_int64(NY), C.c_int64(NSTEP), C.c_double(dt), C.c_double(hx),
            C.c_double(hy), _d(sigma), _d(tau), _d(vp), C.c_int64(len(srci)), _i(srci),
            _i(srcj), _d(srcv), C.c_int64(len(rcvi)), _i(rcvi), _i(rcvj), _d(obs), _d(g)]
    if want_src:
        assert not use_ref
        gs = np.empty((NSTEP, len(srci)))
        f = lib().orc_acoustic_gradient_src
        f.restype = C.c_double
        loss = f(*args, _d(gs), C.c_int(variant))
        return loss, g, gs
    f = ref().ref_acoustic_gradient if use_ref else lib().orc_acoustic_gradient
    f.restype = C.c_double
    if use_ref:
        assert variant == 0
        loss = f(*args)
    else:
        loss = f(*args, C.c_int(variant))
    return loss, g


# ---------------------------------------------------------------- elastic

def elastic_cpml(NX, NY, dx, dy, dt, npml, vp_ref, f0, npower=2.0, k_max=1.0,
                 alpha_max=None, Rcoef=0.001, use_pml=15):
    """ALPHA_MAX_PML defaults to 2*pi*(f0/2) as src/Struct.jl:25."""
    if alpha_max is None:
        alpha_max = 2.0 * np.pi * (f0 / 2.0)
    ax, bx, kx = np.empty(2 * NX), np.empty(2 * NX), np.empty(2 * NX)
    ay, by, ky = np.empty(2 * NY), np.empty(2 * NY), np.empty(2 * NY)
    lib().orc_elastic_cpml(C.c_int64(NX), C.c_int64(NY), C.c_double(dx), C.c_double(dy),
                           C.c_double(dt), C.c_int64(npml), C.c_double(npower),
                           C.c_double(k_max), C.c_double(alpha_max), C.c_double(vp_ref),
                           C.c_double(Rcoef), C.c_int(use_pml), _d(ax), _d(bx), _d(kx),
                           _d(ay), _d(by), _d(ky))
    return ax, bx, kx, ay, by, ky


def elastic_step_fwd(state, lam, mu, rho, ax, bx, ay, by, dt, dx, dy, NX, NY,
                     srci=(), srcj=(), srctype=(), srcv=()):
    state = _f64(state).reshape(-1)
    out = np.empty_like(state)
    srci, srcj, srctype = map(_i64, (srci, srcj, srctype))
    srcv = _f64(srcv)
    lam, mu, rho, ax, bx, ay, by = map(_f64, (lam, mu, rho, ax, bx, ay, by))
    lib().orc_elastic_step_fwd(_d(state), _d(out), _d(lam), _d(mu), _d(rho), _d(ax), _d(bx),
                               _d(ay), _d(by), C.c_double(dt), C.c_double(dx),
                               C.c_double(dy), C.c_int64(NX), C.c_int64(NY),
                               C.c_int64(len(srci)), _i(srci), _i(srcj), _i(srctype),
                               _d(srcv))
    return out


def elastic_step_bwd(state, gout, lam, mu, rho, ax, bx, ay, by, dt, dx, dy, NX, NY):
    N = (NX + 2) * (NY + 2)
    state, gout = _f64(state).reshape(-1), _f64(gout).reshape(-1)
    gin = np.empty_like(state)
    gl, gm, gr = np.zeros(N), np.zeros(N), np.zeros(N)
    lam, mu, rho, ax, bx, ay, by = map(_f64, (lam, mu, rho, ax, bx, ay, by))
    lib().orc_elastic_step_bwd(_d(state), _d(gout), _d(gin), _d(gl), _d(gm), _d(gr),
                               _d(lam), _d(mu), _d(rho), _d(ax), _d(bx), _d(ay), _d(by),
                               C.c_double(dt), C.c_double(dx), C.c_double(dy),
                               C.c_int64(NX), C.c_int64(NY))
    return gin, gl, gm, gr


def elastic_forward(NX, NY, NSTEP, dt, dx, dy, ax, bx, ay, by, lam, mu, rho, srci, srcj,
                    srctype, srcv, rcvi, rcvj, rcvtype, keep_history=False):
    N = (NX + 2) * (NY + 2)
    srci, srcj, srctype, rcvi, rcvj, rcvtype = map(_i64, (srci, srcj, srctype, rcvi, rcvj,
                                                          rcvtype))
    srcv = _f64(srcv).reshape(-1)
    lam, mu, rho, ax, bx, ay, by = map(_f64, (lam, mu, rho, ax, bx, ay, by))
    nrcv = len(rcvi)
    rcvv = np.zeros(nrcv * (NSTEP + 1))
    hist = np.empty((NSTEP + 1) * 13 * N) if keep_history else None
    lib().orc_elastic_forward(C.c_int64(NX), C.c_int64(NY), C.c_int64(NSTEP), C.c_double(dt),
                              C.c_double(dx), C.c_double(dy), _d(ax), _d(bx), _d(ay), _d(by),
                              _d(lam), _d(mu), _d(rho), C.c_int64(len(srci)), _i(srci),
                              _i(srcj), _i(srctype), _d(srcv), C.c_int64(nrcv), _i(rcvi),
                              _i(rcvj), _i(rcvtype), _d(rcvv), _d(hist))
    rcvv = rcvv.reshape(nrcv, NSTEP + 1)
    if keep_history:
        return rcvv, hist.reshape(NSTEP + 1, 13, NX + 2, NY + 2)
    return rcvv


def elastic_gradient(NX, NY, NSTEP, dt, dx, dy, ax, bx, ay, by, lam, mu, rho, srci, srcj,
                     srctype, srcv, rcvi, rcvj, rcvtype, obs, want_src=False):
    """(loss, grad_lambda, grad_mu, grad_rho), plus grad_srcv (NSTEP, nsrc) with
    want_src."""
    N = (NX + 2) * (NY + 2)
    srci, srcj, srctype, rcvi, rcvj, rcvtype = map(_i64, (srci, srcj, srctype, rcvi, rcvj,
                                                          rcvtype))
    srcv, obs = _f64(srcv).reshape(-1), _f64(obs).reshape(-1)
    lam, mu, rho, ax, bx, ay, by = map(_f64, (lam, mu, rho, ax, bx, ay, by))
    gl, gm, gr = np.empty(N), np.empty(N), np.empty(N)
    gs = np.zeros((NSTEP, len(srci)))
    f = lib().orc_elastic_gradient_src
    f.restype = C.c_double
    loss = f(C.c_int64(NX), C.c_int64(NY), C.c_int64(NSTEP), C.c_double(dt), C.c_double(dx),
             C.c_double(dy), _d(ax), _d(bx), _d(ay), _d(by), _d(lam), _d(mu), _d(rho),
             C.c_int64(len(srci)), _i(srci), _i(srcj), _i(srctype), _d(srcv),
             C.c_int64(len(rcvi)), _i(rcvi), _i(rcvj), _i(rcvtype), _d(obs), _d(gl), _d(gm),
             _d(gr), _d(gs) if want_src else None)
    return (loss, gl, gm, gr, gs) if want_src else (loss, gl, gm, gr)


def add_source_fwd(in5, srci, srcj, srctype, srcv, NX, NY, use_ref=False):
    in5 = _f64(in5).reshape(-1)
    out = np.empty_like(in5)
    srci, srcj, srctype = map(_i64, (srci, srcj, srctype))
    srcv = _f64(srcv)
    f = ref().ref_add_source_fwd if use_ref else lib().orc_add_source_fwd
    f(_d(out), _d(in5), C.c_int64(len(srci)), _i(srci), _i(srcj), _i(srctype), _d(srcv),
      C.c_int64(NX), C.c_int64(NY))
    return out


def add_source_bwd(gout5, srci, srcj, srctype, NX, NY, use_ref=False):
    gout5 = _f64(gout5).reshape(-1)
    gin = np.empty_like(gout5)
    srci, srcj, srctype = map(_i64, (srci, srcj, srctype))
    gs = np.zeros(len(srci))
    f = ref().ref_add_source_bwd if use_ref else lib().orc_add_source_bwd
    f(_d(gin), _d(gs), _d(gout5), C.c_int64(len(srci)), _i(srci), _i(srcj), _i(srctype),
      C.c_int64(NX), C.c_int64(NY))
    return gin, gs


def get_receive_fwd(fields5, rcvi, rcvj, rcvtype, NX, NY, use_ref=False):
    """fields5: sequence of five (nt, N) arrays vx, vy, sxx, syy, sxy."""
    fs = [_f64(f).reshape(-1) for f in fields5]
    N = (NX + 2) * (NY + 2)
    nt = fs[0].size // N
    rcvi, rcvj, rcvtype = map(_i64, (rcvi, rcvj, rcvtype))
    out = np.zeros(len(rcvi) * nt)
    if use_ref:
        ref().ref_get_receive_fwd(_d(out), *[_d(f) for f in fs], C.c_int64(nt),
                                  C.c_int64(len(rcvi)), _i(rcvi), _i(rcvj), _i(rcvtype),
                                  C.c_int64(NX), C.c_int64(NY))
    else:
        arr = (_dp * 5)(*[_d(f) for f in fs])
        lib().orc_get_receive_fwd(_d(out), arr, C.c_int64(nt), C.c_int64(len(rcvi)),
                                  _i(rcvi), _i(rcvj), _i(rcvtype), C.c_int64(NX),
                                  C.c_int64(NY))
    return out.reshape(len(rcvi), nt)


def get_receive_bwd(gout, nt, rcvi, rcvj, rcvtype, NX, NY, use_ref=False):
    N = (NX + 2) * (NY + 2)
    gout = _f64(gout).reshape(-1)
    gs = [np.empty(nt * N) for _ in range(5)]
    rcvi, rcvj, rcvtype = map(_i64, (rcvi, rcvj, rcvtype))
    if use_ref:
        ref().ref_get_receive_bwd(*[_d(g) for g in gs], _d(gout), C.c_int64(nt),
                                  C.c_int64(len(rcvi)), _i(rcvi), _i(rcvj), _i(rcvtype),
                                  C.c_int64(NX), C.c_int64(NY))
    else:
        arr = (_dp * 5)(*[_d(g) for g in gs])
        lib().orc_get_receive_bwd(arr, _d(gout), C.c_int64(nt), C.c_int64(len(rcvi)),
                                  _i(rcvi), _i(rcvj), _i(rcvtype), C.c_int64(NX),
                                  C.c_int64(NY))
    return [g.reshape(nt, N) for g in gs]
