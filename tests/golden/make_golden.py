"""Generate the golden fixtures in this directory.

Acoustic step / loop / gradient and the AddSource, GetReceive, ScatterAdd,
Gather fixtures come from the reference's OWN CPU operators compiled from the
reference checkout (oracle/_ref, `make -C oracle ref`).  The elastic fixtures
come from the oracle's restatement of src/Core.jl (the reference has no
compiled elastic stencil).  Run from the repository root, with
ADS_REFERENCE_SRC naming the reference checkout:

    ADS_REFERENCE_SRC=<checkout> python tests/golden/make_golden.py
"""
import os
import sys

import numpy as np

ROOT = os.path.dirname(os.path.dirname(os.path.dirname(os.path.abspath(__file__))))
sys.path.insert(0, ROOT)
import oracle  # noqa: E402

OUT = os.path.dirname(os.path.abspath(__file__))


def acoustic_step():
    # the per-op gradient scripts' setting: 10x10 interior, h = dt = 0.1, random fields
    rng = np.random.default_rng(1234)
    NX, NY = 10, 10
    N = (NX + 2) * (NY + 2)
    ins = [rng.random(N) for _ in range(7)]
    dt, hx, hy = 0.1, 0.1, 0.1
    u, po, qo = oracle.acoustic_step_fwd(*ins, dt, hx, hy, NX, NY, use_ref=True)
    g = [rng.random(N) for _ in range(3)]
    gw, gwo, gp, gq, gc = oracle.acoustic_step_bwd(*g, *ins, dt, hx, hy, NX, NY, u, po, qo,
                                                    use_ref=True)
    np.savez_compressed(os.path.join(OUT, "acoustic_step.npz"), NX=NX, NY=NY, dt=dt, hx=hx,
                        hy=hy, w=ins[0], wold=ins[1], phi=ins[2], psi=ins[3], sigma=ins[4],
                        tau=ins[5], c=ins[6], u=u, phiout=po, psiout=qo, grad_u=g[0],
                        grad_phiout=g[1], grad_psiout=g[2], grad_w=gw, grad_wold=gwo,
                        grad_phi=gp, grad_psi=gq, grad_c=gc)


def acoustic_loop():
    rng = np.random.default_rng(7)
    NX, NY, T = 30, 24, 80
    N = (NX + 2) * (NY + 2)
    dt, h = 1e-3, 10.0
    vp = 2000 + 500 * rng.random(N)
    s, t = oracle.acoustic_pml(NX, NY, h, h, 6, 2000.0)
    srci, srcj = np.array([16, 9]), np.array([8, 12])
    srcv = rng.standard_normal((T, 2)) * 1e3
    rcvi, rcvj = np.arange(5, 26), np.full(21, 4)
    rcvv = oracle.acoustic_forward(NX, NY, T, dt, h, h, s, t, vp, srci, srcj, srcv, rcvi,
                                   rcvj, use_ref=True)
    obs = rcvv * 0.9 + 0.01 * rng.standard_normal(rcvv.shape) * np.abs(rcvv).max()
    loss, grad = oracle.acoustic_gradient(NX, NY, T, dt, h, h, s, t, vp, srci, srcj, srcv,
                                          rcvi, rcvj, obs, use_ref=True)
    np.savez_compressed(os.path.join(OUT, "acoustic_loop.npz"), NX=NX, NY=NY, NSTEP=T, dt=dt,
                        h=h, npml=6, vp_ref=2000.0, vp=vp, sigma=s, tau=t, srci=srci,
                        srcj=srcj, srcv=srcv, rcvi=rcvi, rcvj=rcvj, rcvv=rcvv, obs=obs,
                        loss=loss, grad_vp=grad)


def index_ops():
    rng = np.random.default_rng(5)
    NX, NY = 9, 11
    N = (NX + 2) * (NY + 2)
    srci = np.array([2, 5, 5, 10, 1]); srcj = np.array([3, 7, 7, 12, 1])
    srct = np.array([0, 2, 3, 4, 1]); srcv = rng.standard_normal(5)
    in5 = rng.standard_normal(5 * N)
    out5 = oracle.add_source_fwd(in5, srci, srcj, srct, srcv, NX, NY, use_ref=True)
    g5 = rng.standard_normal(5 * N)
    gin5, gsrc = oracle.add_source_bwd(g5, srci, srcj, srct, NX, NY, use_ref=True)
    nt = 6
    f5 = [rng.standard_normal((nt, N)) for _ in range(5)]
    rcvi = np.array([1, 4, 4, 11, 6, 3]); rcvj = np.array([1, 2, 2, 13, 5, 9])
    rcvt = np.array([0, 1, 1, 2, 3, 4])
    rec = oracle.get_receive_fwd(f5, rcvi, rcvj, rcvt, NX, NY, use_ref=True)
    gout = rng.standard_normal(len(rcvi) * nt)
    grec = oracle.get_receive_bwd(gout, nt, rcvi, rcvj, rcvt, NX, NY, use_ref=True)
    np.savez_compressed(os.path.join(OUT, "index_ops.npz"), NX=NX, NY=NY, srci=srci,
                        srcj=srcj, srctype=srct, srcv=srcv, in5=in5, out5=out5, g5=g5,
                        gin5=gin5, grad_srcv=gsrc, nt=nt, f5=np.stack(f5), rcvi=rcvi,
                        rcvj=rcvj, rcvtype=rcvt, rec=rec, gout=gout, grec=np.stack(grec))


def elastic_small():
    rng = np.random.default_rng(3)
    NX, NY, T = 28, 22, 60
    N = (NX + 2) * (NY + 2)
    dt, dx, dy = 1e-3, 10.0, 12.0
    vp = 3000 + 500 * rng.random(N)
    vs = vp / np.sqrt(3)
    rho = 2000 + 300 * rng.random(N)
    mu = rho * vs * vs
    lam = rho * vp * vp - 2 * mu
    ax, bx, kx, ay, by, ky = oracle.elastic_cpml(NX, NY, dx, dy, dt, 6, 3000.0, 10.0)
    srci, srcj, srct = np.array([15, 15]), np.array([10, 10]), np.array([2, 3])
    srcv = np.repeat(rng.standard_normal((T, 1)) * 1e6, 2, axis=1)
    rcvi = np.concatenate([np.arange(5, 25)] * 2)
    rcvj = np.full(40, 5)
    rcvt = np.array([0] * 20 + [1] * 20)
    rcvv = oracle.elastic_forward(NX, NY, T, dt, dx, dy, ax, bx, ay, by, lam, mu, rho, srci,
                                  srcj, srct, srcv, rcvi, rcvj, rcvt)
    obs = rcvv * 0.8
    loss, gl, gm, gr = oracle.elastic_gradient(NX, NY, T, dt, dx, dy, ax, bx, ay, by, lam,
                                               mu, rho, srci, srcj, srct, srcv, rcvi, rcvj,
                                               rcvt, obs)
    np.savez_compressed(os.path.join(OUT, "elastic_small.npz"), NX=NX, NY=NY, NSTEP=T, dt=dt,
                        dx=dx, dy=dy, npml=6, vp_ref=3000.0, f0=10.0, lam=lam, mu=mu, rho=rho,
                        ax=ax, bx=bx, ay=ay, by=by, srci=srci, srcj=srcj, srctype=srct,
                        srcv=srcv, rcvi=rcvi, rcvj=rcvj, rcvtype=rcvt, rcvv=rcvv, obs=obs,
                        loss=loss, grad_lambda=gl, grad_mu=gm, grad_rho=gr)


if __name__ == "__main__":
    oracle.build(ref=True)
    assert oracle.ref_available(), "the reference checkout is needed to build oracle/_ref"
    acoustic_step()
    acoustic_loop()
    index_ops()
    elastic_small()
    print("golden fixtures written to", OUT)
