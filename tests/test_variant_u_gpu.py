"""Variant U through the batched plans: one_step of src/Core.jl:528-549 (phi
and psi from the new field, the reference's default PropagatorKernel = 0)
against the oracle's restatement of that form, for traces, loss, velocity
gradient and source-time gradient; uneven batches with sources inside the PML
and next to it (the pre-pass subtracts their values), duplicate sources,
checkpoint spacings, resident segments, graphs on and off.  FP64 within
rel-L2 1e-12, FP32 within 1e-5 (traces) and 1e-4 (loss and gradients)."""
import numpy as np
import pytest
import torch

pytestmark = pytest.mark.gpu

U = 1  # ADS_VARIANT_U; the oracle's variant 1 is the same form
TOL64, TOL32, TOL32_TR = 1e-12, 1e-4, 1e-5


def rel(a, b):
    a, b = np.asarray(a, dtype=np.float64), np.asarray(b, dtype=np.float64)
    return np.linalg.norm(a - b) / max(np.linalg.norm(b), 1e-300)


def T(x, dev, dtype=torch.float64):
    return torch.as_tensor(np.asarray(x), dtype=dtype, device=dev)


def pml_case(seed, MX=72, MY=35, nshots=4, npml=5):
    """Uneven shots; shot 0 has sources in the PML corner, on the PML's inner
    edge and two on one cell, so the pre-pass's source terms are exercised."""
    rng = np.random.default_rng(seed)
    shots = []
    for s in range(nshots):
        nx = int(rng.integers(24, 52))
        x0 = int(rng.integers(0, MX - nx + 1))
        nstep = int(rng.integers(35, 80))
        if s == 0:
            srci = np.array([3, npml + 2, 14, 14, nx])
            srcj = np.array([3, 11, npml + 2, npml + 2, MY - 1])
        else:
            n = int(rng.integers(1, 3))
            srci, srcj = rng.integers(2, nx + 2, n), rng.integers(2, MY + 2, n)
        nrcv = int(rng.integers(5, nx - 2))
        rcvi = rng.integers(1, nx + 3, nrcv)
        rcvj = rng.integers(1, MY + 3, nrcv)
        rcvi[0], rcvj[0] = srci[0], srcj[0]  # a receiver on a source cell
        shots.append(dict(x0=x0, nx=nx, nstep=nstep, srci=srci, srcj=srcj,
                          srcv=rng.standard_normal((nstep, len(srci))) * 1e3, rcvi=rcvi,
                          rcvj=rcvj))
    vp = 1800 + 900 * rng.random((MX + 2, MY + 2))
    return MX, MY, shots, vp


def oracle_u(orc, MY, shots, vp, h, dt, npml, vp_ref, obs=None, want_src=False):
    traces, loss, grad, gsrc = [], 0.0, np.zeros_like(vp), []
    for k, s in enumerate(shots):
        nx = s["nx"]
        win = vp[s["x0"]:s["x0"] + nx + 2].reshape(-1)
        sx, ty = orc.acoustic_pml(nx, MY, h, h, npml, vp_ref)
        args = (nx, MY, s["nstep"], dt, h, h, sx, ty, win, s["srci"], s["srcj"], s["srcv"],
                s["rcvi"], s["rcvj"])
        if obs is None:
            traces.append(orc.acoustic_forward(*args, variant=U))
            continue
        out = orc.acoustic_gradient(*args, obs[k], variant=U, want_src=want_src)
        loss += out[0]
        grad[s["x0"]:s["x0"] + nx + 2] += out[1].reshape(nx + 2, MY + 2)
        if want_src:
            gsrc.append(out[2])
    if obs is None:
        return traces
    return (loss, grad, gsrc) if want_src else (loss, grad)


H, DT, NPML, VREF = 10.0, 1e-3, 5, 1500.0


@pytest.fixture(scope="module")
def case(orc):
    MX, MY, shots, vp = pml_case(5)
    ref_tr = oracle_u(orc, MY, shots, vp, H, DT, NPML, VREF)
    rng = np.random.default_rng(6)
    obs = [t * 0.93 + 1e-3 * rng.standard_normal(t.shape) for t in ref_tr]
    ref = oracle_u(orc, MY, shots, vp, H, DT, NPML, VREF, obs, want_src=True)
    return MX, MY, shots, vp, ref_tr, obs, ref


@pytest.mark.parametrize("precision", ["f64", "f32"])
@pytest.mark.parametrize("ckpt,resident,graph", [(13, -1, True), (13, 0, True),
                                                  (13, 2, False), (0, -1, True),
                                                  (1, -1, False), (7, 1, True)])
def test_plan_variant_u_vs_oracle(ads, cuda, case, precision, ckpt, resident, graph):
    MX, MY, shots, vp, ref_tr, obs, (ref_loss, ref_grad, ref_src) = case
    plan = ads.AcousticPlan(MX, MY, H, H, DT, shots, npml=NPML, vp_ref=VREF,
                            precision=precision, ckpt_every=ckpt, resident_segments=resident,
                            use_graph=graph, variant=U)
    tol, tol_tr = (TOL64, TOL64) if precision == "f64" else (TOL32, TOL32_TR)
    got = plan.split_traces(plan.forward(T(vp, cuda)))
    for a, b in zip(got, ref_tr):
        assert rel(a.double().cpu().numpy(), b) <= tol_tr
    loss, grad, gsrc = plan.gradient(T(vp, cuda), plan.pack([T(o, cuda) for o in obs]),
                                     want_source_grad=True)
    torch.cuda.synchronize()
    assert abs(float(loss) - ref_loss) <= tol * ref_loss
    assert rel(grad.cpu().numpy(), ref_grad) <= tol
    for a, b in zip(gsrc, ref_src):
        assert rel(a.cpu().numpy(), b) <= tol
    plan.close()


@pytest.mark.parametrize("precision", ["f64", "f32"])
def test_autotuned_variant_u_plan_vs_oracle(ads, cuda, case, precision):
    MX, MY, shots, vp, ref_tr, obs, (ref_loss, ref_grad, _) = case
    plan = ads.AcousticPlan(MX, MY, H, H, DT, shots, npml=NPML, vp_ref=VREF,
                            precision=precision, ckpt_every=11, autotune=True, variant=U)
    loss, grad = plan.gradient(T(vp, cuda), plan.pack([T(o, cuda) for o in obs]))
    torch.cuda.synchronize()
    tol = TOL64 if precision == "f64" else TOL32
    assert abs(float(loss) - ref_loss) <= tol * ref_loss
    assert rel(grad.cpu().numpy(), ref_grad) <= tol
    plan.close()


def test_variant_u_is_not_variant_w(ads, cuda, case):
    """The two forms differ by a few percent in the PML (the flag is live)."""
    MX, MY, shots, vp, ref_tr, _, _ = case
    trs = []
    for v in (0, U):
        plan = ads.AcousticPlan(MX, MY, H, H, DT, shots, npml=NPML, vp_ref=VREF,
                                precision="f64", variant=v)
        trs.append(plan.forward(T(vp, cuda)).cpu().numpy())
        plan.close()
    assert rel(trs[0], trs[1]) > 1e-4
    assert rel(trs[1], np.concatenate([t.reshape(-1) for t in ref_tr])) <= TOL64


def test_variant_u_rejects_time_blocking(ads, cuda, case):
    MX, MY, shots, vp, _, _, _ = case
    with pytest.raises(ads.AdsError, match="time blocking"):
        ads.AcousticPlan(MX, MY, H, H, DT, shots, npml=NPML, vp_ref=VREF, precision="f32",
                         steps_per_block=4, variant=U)


def test_julia_api_with_the_default_propagator_kernel(ads, orc, cuda):
    """compute_forward_GPU and compute_loss_and_grads_GPU with the reference's
    default PropagatorKernel = 0 run the plans in variant U."""
    rng = np.random.default_rng(9)
    NX, NY, nt = 46, 30, 70
    p = ads.AcousticPropagatorParams(NX=NX, NY=NY, NSTEP=nt, DELTAX=H, DELTAY=H, DELTAT=DT,
                                     NPOINTS_PML=6, vp_ref=VREF)
    assert p.PropagatorKernel == 0
    vp = 1900 + 700 * rng.random((NX + 2, NY + 2))
    srcs = [ads.AcousticSource(np.array([8, 30]), np.array([9, 4]),
                               rng.standard_normal((nt, 2)) * 1e3) for _ in range(2)]
    rcvs = [ads.AcousticReceiver(np.arange(5, 40), np.full(35, 5)) for _ in range(2)]
    sx, ty = orc.acoustic_pml(NX, NY, H, H, 6, VREF)
    ref = [orc.acoustic_forward(NX, NY, nt, DT, H, H, sx, ty, vp.reshape(-1), s.srci, s.srcj,
                                s.srcv, r.rcvi, r.rcvj, variant=U) for s, r in zip(srcs, rcvs)]
    got = ads.compute_forward_GPU(p, srcs, rcvs, vp)
    for a, b in zip(got, ref):
        assert rel(a.cpu().numpy(), b) <= TOL64
    obs = [r * 1.05 for r in ref]
    lref, gref = 0.0, 0.0
    for s, r, o in zip(srcs, rcvs, obs):
        l, g = orc.acoustic_gradient(NX, NY, nt, DT, H, H, sx, ty, vp.reshape(-1), s.srci,
                                     s.srcj, s.srcv, r.rcvi, r.rcvj, o, variant=U)
        lref, gref = lref + l, gref + g
    loss, grad = ads.compute_loss_and_grads_GPU(p, srcs, rcvs, obs, vp)
    assert abs(float(loss) - lref) <= TOL64 * lref
    assert rel(grad.cpu().numpy().reshape(-1), gref) <= TOL64
    # aux_loss (src/Utils.jl:309-311) and the reference's one-GPU lists
    losses, grads = ads.compute_loss_and_grads_GPU(p, srcs, rcvs, obs, vp, aux_loss=2.5,
                                                   as_lists=True)
    assert len(losses) == len(grads) == 1
    assert abs(float(losses[0]) - (lref + 2.5)) <= TOL64 * lref
    assert rel(grads[0].cpu().numpy().reshape(-1), gref) <= TOL64
