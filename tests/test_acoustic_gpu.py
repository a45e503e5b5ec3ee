"""Acoustic parity on the GPU through the C ABI: the single-step drop-in against
the reference's compiled operator (golden, bit-exact), the whole-path FP64
forward/gradient against the oracle (rel-L2 <= 1e-12), FP32 against the FP64
oracle (rel-L2 <= 1e-4 on the gradient), uneven multi-shot batches, edge cases."""
import numpy as np
import pytest
import torch

from conftest import golden

pytestmark = pytest.mark.gpu

TOL64 = 1e-12   # FP64 drop-in vs reference CPU operators (rel-L2)
TOL32 = 1e-4    # FP32 stencils / FP64 accumulation vs FP64 oracle (rel-L2, gradient)


def rel(a, b):
    a, b = np.asarray(a, dtype=np.float64), np.asarray(b, dtype=np.float64)
    return np.linalg.norm(a - b) / max(np.linalg.norm(b), 1e-300)


def T(x, dev, dtype=torch.float64):
    return torch.as_tensor(np.asarray(x), dtype=dtype, device=dev)


def test_step_forward_bitexact_with_reference(ads, cuda):
    g = golden("acoustic_step.npz")
    NX, NY = int(g["NX"]), int(g["NY"])
    ins = [T(g[k], cuda) for k in ("w", "wold", "phi", "psi", "sigma", "tau", "c")]
    u, po, qo = ads.acoustic_one_step(*ins, float(g["dt"]), float(g["hx"]), float(g["hy"]), NX,
                                      NY)
    assert np.array_equal(u.cpu().numpy(), g["u"])
    assert np.array_equal(po.cpu().numpy(), g["phiout"])
    assert np.array_equal(qo.cpu().numpy(), g["psiout"])


def test_step_backward_matches_reference(ads, cuda):
    g = golden("acoustic_step.npz")
    NX, NY = int(g["NX"]), int(g["NY"])
    ins = [T(g[k], cuda) for k in ("w", "wold", "phi", "psi", "sigma", "tau", "c")]
    gs = [T(g[k], cuda) for k in ("grad_u", "grad_phiout", "grad_psiout")]
    outs = [T(g[k], cuda) for k in ("u", "phiout", "psiout")]
    got = ads.acoustic_one_step_grad(*gs, *ins, float(g["dt"]), float(g["hx"]), float(g["hy"]),
                                     NX, NY, *outs)
    for t, k in zip(got, ("grad_w", "grad_wold", "grad_phi", "grad_psi", "grad_c")):
        assert rel(t.cpu().numpy(), g[k]) <= 1e-14, k


@pytest.mark.parametrize("variant", [0, 1])
@pytest.mark.parametrize("shape", [(1, 1), (7, 3), (45, 70)])
def test_step_random_vs_oracle(ads, orc, cuda, variant, shape):
    NX, NY = shape
    N = (NX + 2) * (NY + 2)
    rng = np.random.default_rng(NX * 100 + NY + variant)
    ins = [rng.standard_normal(N) for _ in range(7)]
    ref = orc.acoustic_step_fwd(*ins, 0.01, 0.3, 0.2, NX, NY, variant=variant)
    got = ads.acoustic_one_step(*[T(x, cuda) for x in ins], 0.01, 0.3, 0.2, NX, NY, variant)
    for a, b in zip(got, ref):
        assert rel(a.cpu().numpy(), b) <= 1e-15
    gs = [rng.standard_normal(N) for _ in range(3)]
    refg = orc.acoustic_step_bwd(*gs, *ins, 0.01, 0.3, 0.2, NX, NY, *ref, variant=variant)
    gotg = ads.acoustic_one_step_grad(*[T(x, cuda) for x in gs], *[T(x, cuda) for x in ins],
                                      0.01, 0.3, 0.2, NX, NY, *[T(x, cuda) for x in ref],
                                      variant)
    for a, b in zip(gotg, refg):
        assert rel(a.cpu().numpy(), b) <= 1e-13


def test_step_f32_close_to_f64(ads, orc, cuda):
    NX, NY = 30, 41
    N = (NX + 2) * (NY + 2)
    rng = np.random.default_rng(0)
    ins = [rng.random(N) for _ in range(7)]
    ref = orc.acoustic_step_fwd(*ins, 0.1, 1.0, 1.0, NX, NY)
    got = ads.acoustic_one_step(*[T(x, cuda, torch.float32) for x in ins], 0.1, 1.0, 1.0, NX, NY)
    for a, b in zip(got, ref):
        assert rel(a.double().cpu().numpy(), b) <= 1e-6


def test_autograd_function_matches_oracle(ads, orc, cuda):
    NX, NY = 12, 9
    N = (NX + 2) * (NY + 2)
    rng = np.random.default_rng(5)
    ins = [T(rng.random(N), cuda).requires_grad_(True) for _ in range(7)]
    u, po, qo = ads.AcousticOneStep.apply(*ins, 0.1, 0.5, 0.5, NX, NY, 0)
    wu, wp, wq = (rng.standard_normal(N) for _ in range(3))
    (u * T(wu, cuda) + po * T(wp, cuda) + qo * T(wq, cuda)).sum().backward()
    args = [t.detach().cpu().numpy() for t in ins]
    refo = orc.acoustic_step_fwd(*args, 0.1, 0.5, 0.5, NX, NY)
    refg = orc.acoustic_step_bwd(wu, wp, wq, *args, 0.1, 0.5, 0.5, NX, NY, *refo)
    for t, r in zip((ins[0], ins[1], ins[2], ins[3], ins[6]), refg):
        assert rel(t.grad.cpu().numpy(), r) <= 1e-13


def loop_case(g):
    NX, NY, Tn = int(g["NX"]), int(g["NY"]), int(g["NSTEP"])
    shot = dict(x0=0, nx=NX, nstep=Tn, srci=g["srci"], srcj=g["srcj"], srcv=g["srcv"],
                rcvi=g["rcvi"], rcvj=g["rcvj"])
    return NX, NY, Tn, shot


@pytest.mark.parametrize("use_graph", [True, False])
@pytest.mark.parametrize("ckpt", [0, 1, 7, 79])
@pytest.mark.parametrize("resident", [-1, 0, 2])
def test_plan_fp64_matches_reference_golden(ads, cuda, use_graph, ckpt, resident):
    """resident: checkpoint segments whose wavefields stay on the device
    (-1 none: every segment recomputed; 0 as many as fit: all of them here;
    2 the last two)."""
    g = golden("acoustic_loop.npz")
    NX, NY, Tn, shot = loop_case(g)
    h, dt = float(g["h"]), float(g["dt"])
    plan = ads.AcousticPlan(NX, NY, h, h, dt, [shot], npml=int(g["npml"]),
                            vp_ref=float(g["vp_ref"]), precision="f64", use_graph=use_graph,
                            ckpt_every=ckpt, resident_segments=resident)
    nseg = -(-(Tn - 1) // (ckpt if ckpt else 100 if Tn >= 400 else
                         max(1, int(np.ceil(np.sqrt(Tn) * 2)))))
    assert plan.resident_segments == {-1: 0, 0: nseg, 2: min(2, nseg)}[resident]
    vp = T(g["vp"].reshape(NX + 2, NY + 2), cuda)
    tr = plan.forward(vp)
    assert rel(tr.cpu().numpy(), g["rcvv"].reshape(-1)) <= TOL64
    loss, grad, tr2 = plan.gradient(vp, T(g["obs"].reshape(-1), cuda), want_traces=True)
    torch.cuda.synchronize()
    assert abs(float(loss) - float(g["loss"])) <= TOL64 * float(g["loss"])
    assert rel(grad.cpu().numpy().reshape(-1), g["grad_vp"]) <= TOL64
    assert torch.equal(tr, tr2)
    plan.close()


def test_plan_fp32_vs_fp64_oracle(ads, cuda):
    g = golden("acoustic_loop.npz")
    NX, NY, Tn, shot = loop_case(g)
    h, dt = float(g["h"]), float(g["dt"])
    plan = ads.AcousticPlan(NX, NY, h, h, dt, [shot], npml=int(g["npml"]),
                            vp_ref=float(g["vp_ref"]), precision="f32", ckpt_every=10)
    vp = T(g["vp"].reshape(NX + 2, NY + 2), cuda)
    loss, grad, tr = plan.gradient(vp, T(g["obs"].reshape(-1), cuda, torch.float32),
                                   want_traces=True)
    torch.cuda.synchronize()
    assert rel(tr.double().cpu().numpy(), g["rcvv"].reshape(-1)) <= 1e-5
    assert rel(grad.cpu().numpy().reshape(-1), g["grad_vp"]) <= TOL32
    assert abs(float(loss) - float(g["loss"])) <= 1e-4 * float(g["loss"])
    plan.close()


def uneven_case(seed, MX=70, MY=33, nshots=5, precision_rows=None):
    rng = np.random.default_rng(seed)
    shots = []
    for s in range(nshots):
        nx = int(rng.integers(20, 50))
        x0 = int(rng.integers(0, MX - nx + 1))
        nstep = int(rng.integers(30, 90))
        nsrc = int(rng.integers(0, 3)) if s else 1
        nrcv = int(rng.integers(0, nx - 2)) if s != 1 else 0
        srci = rng.integers(2, nx + 2, nsrc)
        srcj = rng.integers(2, MY + 2, nsrc)
        rcvi = rng.integers(1, nx + 3, nrcv)
        rcvj = rng.integers(1, MY + 3, nrcv)
        if nrcv > 3:  # duplicate receivers and a frame receiver
            rcvi[1], rcvj[1] = rcvi[0], rcvj[0]
            rcvi[2] = 1
        if nsrc == 2:  # two sources on one cell
            srci[1], srcj[1] = srci[0], srcj[0]
        shots.append(dict(x0=x0, nx=nx, nstep=nstep, srci=srci, srcj=srcj,
                          srcv=rng.standard_normal((nstep, nsrc)) * 1e3, rcvi=rcvi,
                          rcvj=rcvj))
    vp = 1800 + 900 * rng.random((MX + 2, MY + 2))
    return MX, MY, shots, vp


def oracle_multishot(orc, MX, MY, shots, vp, h, dt, npml, vp_ref, obs=None):
    traces, loss, grad = [], 0.0, np.zeros_like(vp)
    for k, s in enumerate(shots):
        nx = s["nx"]
        win = vp[s["x0"]:s["x0"] + nx + 2].reshape(-1)
        sx, ty = orc.acoustic_pml(nx, MY, h, h, npml, vp_ref)
        if obs is None:
            traces.append(orc.acoustic_forward(nx, MY, s["nstep"], dt, h, h, sx, ty, win,
                                               s["srci"], s["srcj"], s["srcv"], s["rcvi"],
                                               s["rcvj"]))
        else:
            l, gk = orc.acoustic_gradient(nx, MY, s["nstep"], dt, h, h, sx, ty, win, s["srci"],
                                          s["srcj"], s["srcv"], s["rcvi"], s["rcvj"], obs[k])
            loss += l
            grad[s["x0"]:s["x0"] + nx + 2] += gk.reshape(nx + 2, MY + 2)
    return traces if obs is None else (loss, grad)


@pytest.mark.parametrize("precision", ["f64", "f32"])
@pytest.mark.parametrize("rows", [0, 1, 3])
@pytest.mark.parametrize("resident", [-1, 0, 3])
def test_plan_uneven_multishot_vs_oracle(ads, orc, cuda, precision, rows, resident):
    MX, MY, shots, vp = uneven_case(21)
    h, dt, npml, vref = 10.0, 1e-3, 5, 1500.0
    ref_tr = oracle_multishot(orc, MX, MY, shots, vp, h, dt, npml, vref)
    rng = np.random.default_rng(3)
    obs = [t * 0.95 + 1e-3 * rng.standard_normal(t.shape) for t in ref_tr]
    ref_loss, ref_grad = oracle_multishot(orc, MX, MY, shots, vp, h, dt, npml, vref, obs)
    plan = ads.AcousticPlan(MX, MY, h, h, dt, shots, npml=npml, vp_ref=vref,
                            precision=precision, ckpt_every=13, rows_per_thread=rows,
                            resident_segments=resident)
    dtype = plan.dtype
    tr = plan.forward(T(vp, cuda))
    got = plan.split_traces(tr)
    tol_tr = TOL64 if precision == "f64" else 1e-5
    for a, b in zip(got, ref_tr):
        if b.size:
            assert rel(a.double().cpu().numpy(), b) <= tol_tr
    loss, grad = plan.gradient(T(vp, cuda), plan.pack([T(o, cuda, dtype) for o in obs]))
    torch.cuda.synchronize()
    tol = TOL64 if precision == "f64" else TOL32
    assert abs(float(loss) - ref_loss) <= tol * ref_loss
    assert rel(grad.cpu().numpy(), ref_grad) <= tol
    plan.close()


@pytest.mark.parametrize("kb,rows", [(1, 0), (2, 0), (4, 0), (8, 0), (4, 3), (8, 5)])
def test_plan_fp32_time_blocked_vs_oracle(ads, orc, cuda, kb, rows):
    MX, MY, shots, vp = uneven_case(77, nshots=4)
    h, dt, npml, vref = 10.0, 1e-3, 5, 1500.0
    ref_tr = oracle_multishot(orc, MX, MY, shots, vp, h, dt, npml, vref)
    rng = np.random.default_rng(8)
    obs = [t * 0.9 + 1e-3 * rng.standard_normal(t.shape) for t in ref_tr]
    ref_loss, ref_grad = oracle_multishot(orc, MX, MY, shots, vp, h, dt, npml, vref, obs)
    plan = ads.AcousticPlan(MX, MY, h, h, dt, shots, npml=npml, vp_ref=vref, precision="f32",
                            ckpt_every=7, steps_per_block=kb, block_rows=rows)
    tr = plan.forward(T(vp, cuda))
    for a, b in zip(plan.split_traces(tr), ref_tr):
        if b.size:
            assert rel(a.double().cpu().numpy(), b) <= 1e-5
    loss, grad = plan.gradient(T(vp, cuda), plan.pack([T(o, cuda, torch.float32) for o in obs]))
    torch.cuda.synchronize()
    assert abs(float(loss) - ref_loss) <= TOL32 * ref_loss
    assert rel(grad.cpu().numpy(), ref_grad) <= TOL32
    plan.close()


@pytest.mark.parametrize("precision", ["f64", "f32"])
@pytest.mark.parametrize("resident", [0, -1])
def test_autotuned_plan_vs_oracle(ads, orc, cuda, precision, resident):
    """Tuned row heights; FP32 plans without resident segments also tune the
    forward steps per launch (1, 2 or 4)."""
    MX, MY, shots, vp = uneven_case(31, nshots=5)
    h, dt, npml, vref = 10.0, 1e-3, 5, 1500.0
    ref_tr = oracle_multishot(orc, MX, MY, shots, vp, h, dt, npml, vref)
    obs = [t * 0.97 for t in ref_tr]
    ref_loss, ref_grad = oracle_multishot(orc, MX, MY, shots, vp, h, dt, npml, vref, obs)
    plan = ads.AcousticPlan(MX, MY, h, h, dt, shots, npml=npml, vp_ref=vref, precision=precision,
                            ckpt_every=11, autotune=2, resident_segments=resident)
    assert plan.steps_per_block in ((1, 2, 4) if precision == "f32" and resident < 0 else (1,))
    dtype = plan.dtype
    loss, grad = plan.gradient(T(vp, cuda), plan.pack([T(o, cuda, dtype) for o in obs]))
    torch.cuda.synchronize()
    tol = TOL64 if precision == "f64" else TOL32
    assert abs(float(loss) - ref_loss) <= tol * ref_loss
    assert rel(grad.cpu().numpy(), ref_grad) <= tol
    plan.close()


@pytest.mark.parametrize("rows", [2, 4])
@pytest.mark.parametrize("resident", [-1, 2])
def test_fp64_pml_warp_kinds_vs_oracle(ads, orc, cuda, rows, resident):
    """FP64 plans specialise the PML kernels by warp kind (sigma rows only, tau
    columns only, corners). A 150 x 190 grid with a 12-cell PML holds warps of
    every kind and interior warps inside PML items (64-column forward and
    32-column adjoint strips); the uneven shot windows move the sigma rows
    against the row tiles."""
    MX, MY, npml, h, dt, vref = 150, 190, 12, 10.0, 1e-3, 1500.0
    rng = np.random.default_rng(17)
    shots = []
    for x0, nx, nstep in ((0, 150, 120), (13, 101, 120), (40, 97, 95)):
        shots.append(dict(x0=x0, nx=nx, nstep=nstep, srci=[nx // 2], srcj=[MY // 3],
                          srcv=rng.standard_normal((nstep, 1)) * 1e3,
                          rcvi=np.arange(2, nx + 2, 3), rcvj=np.full(len(range(2, nx + 2, 3)), 20)))
    vp = 1800 + 900 * rng.random((MX + 2, MY + 2))
    ref_tr = oracle_multishot(orc, MX, MY, shots, vp, h, dt, npml, vref)
    obs = [t * 0.95 for t in ref_tr]
    ref_loss, ref_grad = oracle_multishot(orc, MX, MY, shots, vp, h, dt, npml, vref, obs)
    plan = ads.AcousticPlan(MX, MY, h, h, dt, shots, npml=npml, vp_ref=vref, precision="f64",
                            ckpt_every=17, rows_per_thread=rows, resident_segments=resident)
    assert plan.rows == (rows, rows, rows, rows)
    for a, b in zip(plan.split_traces(plan.forward(T(vp, cuda))), ref_tr):
        assert rel(a.cpu().numpy(), b) <= TOL64
    loss, grad = plan.gradient(T(vp, cuda), plan.pack([T(o, cuda) for o in obs]))
    torch.cuda.synchronize()
    assert abs(float(loss) - ref_loss) <= TOL64 * ref_loss
    assert rel(grad.cpu().numpy(), ref_grad) <= TOL64
    plan.close()


def test_repeated_calls_are_deterministic(ads, cuda):
    MX, MY, shots, vp = uneven_case(5, nshots=3)
    plan = ads.AcousticPlan(MX, MY, 10.0, 10.0, 1e-3, shots, npml=5, precision="f32")
    obs = torch.zeros(plan.trace_count, dtype=torch.float32, device=cuda)
    l1, g1 = plan.gradient(T(vp, cuda), obs)
    l2, g2 = plan.gradient(T(vp, cuda), obs)
    assert torch.equal(g1, g2) and float(l1) == float(l2)
    plan.close()


def test_invalid_geometry_rejected(ads, cuda):
    shot = dict(x0=0, nx=10, nstep=20, srci=[1], srcj=[5], srcv=np.zeros((20, 1)),
                rcvi=[3], rcvj=[3])
    with pytest.raises(ads.AdsError, match="interior"):
        ads.AcousticPlan(10, 10, 10.0, 10.0, 1e-3, [shot])
    shot = dict(x0=5, nx=10, nstep=20, srci=[4], srcj=[5], srcv=np.zeros((20, 1)),
                rcvi=[3], rcvj=[3])
    with pytest.raises(ads.AdsError, match="window"):
        ads.AcousticPlan(10, 10, 10.0, 10.0, 1e-3, [shot])
    shot = dict(x0=0, nx=10, nstep=20, srci=[4], srcj=[5], srcv=np.zeros((19, 1)),
                rcvi=[3], rcvj=[3])
    with pytest.raises(ads.AdsError, match="rows"):
        ads.AcousticPlan(10, 10, 10.0, 10.0, 1e-3, [shot])


def test_julia_style_api(ads, orc, cuda):
    """PropagatorKernel 1 (the custom operator's form, on the plans) against the
    reference's golden loop; 0 (one_step: phi / psi from the new u, on the
    single-step operator chain) against the oracle's restatement of it."""
    g = golden("acoustic_loop.npz")
    NX, NY, Tn = int(g["NX"]), int(g["NY"]), int(g["NSTEP"])
    h, dt = float(g["h"]), float(g["dt"])
    src = ads.AcousticSource(g["srci"], g["srcj"], g["srcv"])
    rcv = ads.AcousticReceiver(g["rcvi"], g["rcvj"])
    kw = dict(NX=NX, NY=NY, NSTEP=Tn, DELTAX=h, DELTAY=h, DELTAT=dt,
              NPOINTS_PML=int(g["npml"]), vp_ref=float(g["vp_ref"]))
    p = ads.AcousticPropagatorParams(PropagatorKernel=1, **kw)
    ap = ads.AcousticPropagatorSolver(p, src, g["vp"])
    ads.SimulatedObservation(ap, rcv)
    assert rel(rcv.rcvv.cpu().numpy(), g["rcvv"]) <= TOL64
    loss, grad = ads.compute_loss_and_grads_GPU(p, [src], [rcv], [g["obs"]], g["vp"])
    assert rel(grad.cpu().numpy().reshape(-1), g["grad_vp"]) <= TOL64
    pu = ads.AcousticPropagatorParams(**kw)
    assert pu.PropagatorKernel == 0 and ads.step_variant(pu) == ads.ADS_VARIANT_U
    s, t = orc.acoustic_pml(NX, NY, h, h, int(g["npml"]), float(g["vp_ref"]))
    args = (NX, NY, Tn, dt, h, h, s, t, g["vp"], g["srci"], g["srcj"], g["srcv"], g["rcvi"],
            g["rcvj"])
    ref_tr = orc.acoustic_forward(*args, variant=1)
    ref_loss, ref_grad = orc.acoustic_gradient(*args, g["obs"], variant=1)
    assert rel(ref_tr, g["rcvv"]) > 1e-8  # the two forms differ in the PML
    apu = ads.AcousticPropagatorSolver(pu, src, g["vp"])
    ads.SimulatedObservation(apu, rcv)
    assert rel(rcv.rcvv.cpu().numpy(), ref_tr) <= TOL64
    # the reference's wavefield histories on the propagator (src/Struct.jl:140-147)
    for prop, variant in ((ap, 0), (apu, 1)):
        hist = orc.acoustic_forward(*args, variant=variant, keep_history=True)[1]
        assert tuple(prop.u.shape) == (Tn + 1, NX + 2, NY + 2) == tuple(prop.psi.shape)
        assert rel(prop.u.cpu().numpy(), hist) <= TOL64, variant
    tr = ads.compute_forward_GPU(pu, [src], [rcv], g["vp"])
    assert rel(tr[0].cpu().numpy(), ref_tr) <= TOL64
    loss, grad = ads.compute_loss_and_grads_GPU(pu, [src, src], [rcv, rcv],
                                                [g["obs"], g["obs"]], g["vp"])
    assert abs(float(loss) - 2 * ref_loss) <= TOL64 * 2 * ref_loss
    assert rel(grad.cpu().numpy().reshape(-1), 2 * ref_grad) <= TOL64


def test_dropin_operator_chain_matches_reference_golden(ads, cuda):
    """The per-step FP64 operator chain (step, ScatterAdd, Gather and their
    gradients, full history) reproduces the reference loss and gradient."""
    g = golden("acoustic_loop.npz")
    NX, NY, Tn = int(g["NX"]), int(g["NY"]), int(g["NSTEP"])
    p = ads.AcousticPropagatorParams(NX=NX, NY=NY, NSTEP=Tn, DELTAX=float(g["h"]),
                                     DELTAY=float(g["h"]), DELTAT=float(g["dt"]),
                                     NPOINTS_PML=int(g["npml"]), vp_ref=float(g["vp_ref"]),
                                     PropagatorKernel=1)
    src = ads.AcousticSource(g["srci"], g["srcj"], g["srcv"])
    rcv = ads.AcousticReceiver(g["rcvi"], g["rcvj"])
    loss, grad = ads.dropin_loss_and_grad(p, src, rcv, g["obs"], g["vp"])
    torch.cuda.synchronize()
    assert abs(float(loss) - float(g["loss"])) <= TOL64 * float(g["loss"])
    assert rel(grad.cpu().numpy().reshape(-1), g["grad_vp"]) <= TOL64


def test_dropin_chain_at_the_reference_cpu_case_vs_oracle(ads, orc, cuda):
    """The plain FP64 drop-in at the reference CPU operators' own case: 200 x 200
    interior plus a 20-cell PML, h = 10 m, dt = 1 ms, 1000 steps, a 10 Hz Ricker
    20 cells below the PML, 200 receivers 5 cells below it.  Loss and velocity
    gradient against the oracle (bit-identical to the compiled reference
    operators) within 1e-12."""
    NX = NY = 240
    npml, T, h, dt = 20, 1000, 10.0, 1e-3
    vp = ads.layered_gaussian_model(NX + 2, NY + 2, 2000.0, 3500.0, seed=7)
    vref = float(vp.mean())
    p = ads.AcousticPropagatorParams(NX=NX, NY=NY, NSTEP=T, DELTAX=h, DELTAY=h, DELTAT=dt,
                                     NPOINTS_PML=npml, vp_ref=vref, PropagatorKernel=1)
    wav = ads.Ricker(p, ads.ricker_width_samples(10.0, dt), 1.5 / 10.0 / dt, 1e6)
    src = ads.AcousticSource(np.array([NX // 2 + 1]), np.array([npml + 21]), wav[:, None])
    rcv = ads.AcousticReceiver(np.arange(npml + 2, npml + 202), np.full(200, npml + 6))
    s, t = orc.acoustic_pml(NX, NY, h, h, npml, vref)
    args = (NX, NY, T, dt, h, h, s, t)
    obs = orc.acoustic_forward(*args, (vp * 1.01).reshape(-1), src.srci, src.srcj, src.srcv,
                               rcv.rcvi, rcv.rcvj)
    ref_loss, ref_grad = orc.acoustic_gradient(*args, vp.reshape(-1), src.srci, src.srcj,
                                               src.srcv, rcv.rcvi, rcv.rcvj, obs)
    loss, grad = ads.dropin_loss_and_grad(p, src, rcv, obs, vp)
    torch.cuda.synchronize()
    assert abs(float(loss) - ref_loss) <= TOL64 * ref_loss
    assert rel(grad.cpu().numpy().reshape(-1), ref_grad) <= TOL64


@pytest.mark.parametrize("precision,tol", [("f64", TOL64), ("f32", 1e-4)])
@pytest.mark.parametrize("resident", [-1, 0])
def test_source_time_gradient_vs_oracle(ads, orc, cuda, precision, tol, resident):
    """d loss / d srcv from the plan's adjoint (two shots of different length
    and source count, one source on a receiver's cell) against the oracle."""
    rng = np.random.default_rng(11)
    NX, NY, h, dt, npml = 40, 36, 10.0, 1e-3, 8
    N = (NX + 2) * (NY + 2)
    vp = 2000 + 400 * rng.random(N)
    s, t = orc.acoustic_pml(NX, NY, h, h, npml, 2000.0)
    rcvi, rcvj = np.arange(10, 34), np.full(24, 12)
    cases = [dict(nstep=70, srci=[20, 15], srcj=[20, 12]), dict(nstep=55, srci=[25], srcj=[18])]
    shots, obs, want = [], [], []
    for c in cases:
        nt = c["nstep"]
        srcv = rng.standard_normal((nt, len(c["srci"]))) * 1e4
        o = orc.acoustic_forward(NX, NY, nt, dt, h, h, s, t, vp * 1.04, c["srci"], c["srcj"],
                                 srcv, rcvi, rcvj)
        _, _, gs = orc.acoustic_gradient(NX, NY, nt, dt, h, h, s, t, vp, c["srci"], c["srcj"],
                                         srcv, rcvi, rcvj, o, want_src=True)
        shots.append(dict(x0=0, nx=NX, nstep=nt, srci=c["srci"], srcj=c["srcj"], srcv=srcv,
                          rcvi=rcvi, rcvj=rcvj))
        obs.append(T(o.reshape(-1), cuda))
        want.append(gs)
    plan = ads.AcousticPlan(NX, NY, h, h, dt, shots, npml=npml, vp_ref=2000.0,
                            precision=precision, ckpt_every=16, resident_segments=resident)
    out = plan.gradient(T(vp.reshape(NX + 2, NY + 2), cuda), plan.pack(obs),
                        want_source_grad=True)
    torch.cuda.synchronize()
    got = out[-1]
    for k in range(len(cases)):
        g = got[k].cpu().numpy()
        assert g.shape == want[k].shape
        assert np.all(g[0] == 0.0)
        assert rel(g, want[k]) <= tol, (k, rel(g, want[k]))
    plan.close()


@pytest.mark.parametrize("precision,tol", [("f64", TOL64), ("f32", 1e-4)])
def test_location_gradient_of_gaussian_source_vs_oracle(ads, orc, cuda, precision, tol):
    """A Gaussian variable source (a source on every interior cell,
    src/Utils.jl:603-633) through a plan: d loss / d srcv against the oracle,
    then the location gradient d loss / d (x, y) and d loss / d v from it."""
    rng = np.random.default_rng(13)
    NX, NY, h, dt, npml, nt = 40, 36, 10.0, 1e-3, 8, 60
    p = ads.AcousticPropagatorParams(NX=NX, NY=NY, NSTEP=nt, DELTAX=h, DELTAY=h, DELTAT=dt)
    vp = 2000 + 400 * rng.random((NX + 2) * (NY + 2))
    s, t = orc.acoustic_pml(NX, NY, h, h, npml, 2000.0)
    rcvi, rcvj = np.arange(10, 34), np.full(24, 12)
    v = ads.Ricker(p, 5.0, 15.0) * 1e5
    x, y = 203.0, 177.0
    i, j, srcv = ads.variable_source(p, x, y, v, sigma=1.3)
    o = orc.acoustic_forward(NX, NY, nt, dt, h, h, s, t, vp * 1.04, i, j, srcv, rcvi, rcvj)
    _, _, G = orc.acoustic_gradient(NX, NY, nt, dt, h, h, s, t, vp, i, j, srcv, rcvi, rcvj, o,
                                    want_src=True)
    plan = ads.AcousticPlan(NX, NY, h, h, dt, [dict(x0=0, nx=NX, nstep=nt, srci=i, srcj=j,
                                                    srcv=srcv, rcvi=rcvi, rcvj=rcvj)],
                            npml=npml, vp_ref=2000.0, precision=precision, ckpt_every=16)
    out = plan.gradient(T(vp.reshape(NX + 2, NY + 2), cuda), plan.pack([T(o.reshape(-1), cuda)]),
                        want_source_grad=True)
    torch.cuda.synchronize()
    got = out[-1][0]
    assert got.shape == G.shape and rel(got.cpu().numpy(), G) <= tol
    gx, gy, gv = ads.variable_source_grad(p, x, y, v, got, sigma=1.3)
    wx, wy, wv = ads.variable_source_grad(p, x, y, v, G, sigma=1.3)
    # (x, y) sums G against weights of both signs: FP32 is held to 1e-3 there
    txy = tol if precision == "f64" else 1e-3
    assert np.hypot(gx - wx, gy - wy) <= txy * np.hypot(wx, wy), (gx, wx, gy, wy)
    assert gv.device == got.device and rel(gv.cpu().numpy(), wv) <= tol
    plan.close()


@pytest.mark.parametrize("precision", ["f64", "f32"])
def test_set_source_values_matches_a_fresh_plan(ads, cuda, precision):
    """Wavelets replaced in place (uneven shots, so the plan's internal shot
    order differs from the caller's; some shots without sources) give
    bitwise the traces, loss and gradients of a plan created with them."""
    MX, MY, shots, vp = uneven_case(21)
    h, dt, npml, vref = 10.0, 1e-3, 5, 1500.0
    kw = dict(npml=npml, vp_ref=vref, precision=precision, ckpt_every=13)
    a = ads.AcousticPlan(MX, MY, h, h, dt, shots, **kw)
    zeroed = [dict(s, srcv=np.zeros_like(s["srcv"])) for s in shots]
    b = ads.AcousticPlan(MX, MY, h, h, dt, zeroed, **kw)
    assert any(len(s["srci"]) == 0 for s in shots) and len({s["nstep"] for s in shots}) > 1
    for k, s in enumerate(shots):
        b.set_source_values(k, T(s["srcv"], cuda))
    ta, tb = a.forward(T(vp, cuda)), b.forward(T(vp, cuda))
    assert torch.equal(ta, tb)
    obs = ta * 0.9
    ra = a.gradient(T(vp, cuda), obs, want_source_grad=True)
    rb = b.gradient(T(vp, cuda), obs, want_source_grad=True)
    torch.cuda.synchronize()
    assert torch.equal(ra[0], rb[0]) and torch.equal(ra[1], rb[1])
    assert all(torch.equal(x, y) for x, y in zip(ra[2], rb[2]))
    with pytest.raises(ads.AdsError):
        b.set_source_values(-1, T(shots[0]["srcv"], cuda))
    a.close()
    b.close()


def test_source_lbfgs_on_the_plan(ads, cuda):
    """The source location / wavelet inversion loop on an FP64 plan: a
    misplaced Gaussian source moves back onto the one that made the data."""
    rng = np.random.default_rng(21)
    NX, NY, h, dt, npml, nt = 40, 36, 10.0, 1e-3, 8, 120
    p = ads.AcousticPropagatorParams(NX=NX, NY=NY, NSTEP=nt, DELTAX=h, DELTAY=h, DELTAT=dt)
    vp = 2000 + 300 * rng.random((NX + 2, NY + 2))
    v = ads.Ricker(p, 4.0, 15.0)
    i, j, sv = ads.variable_source(p, 203.0, 186.0, v * 1e3, sigma=0.5)
    shot = dict(x0=0, nx=NX, nstep=nt, srci=i, srcj=j, srcv=sv, rcvi=np.arange(10, 34),
                rcvj=np.full(24, 12))
    plan = ads.AcousticPlan(NX, NY, h, h, dt, [shot], npml=npml, vp_ref=2000.0,
                            precision="f64", ckpt_every=20)
    obs = plan.forward(T(vp, cuda)).clone()
    x, y, vv, losses = ads.source_lbfgs(plan, p, T(vp, cuda), obs, 216.0, 175.0, 0.8 * v,
                                        sigma=0.5, source_scale=1e3, max_iter=60)
    # the oracle in place of the plan: 1.3e-3 and 0.017 after 50 iterations
    assert losses[-1] < 1e-2 * losses[0], losses
    assert np.hypot(x - 203.0, y - 186.0) < 0.1 * np.hypot(13.0, 11.0), (x, y)
    plan.close()


def test_compute_forward_GPU_matches_the_golden_traces(ads, cuda):
    """compute_forward_GPU (src/Utils.jl:574-601): every shot's traces from
    one batched plan, against the reference's golden traces."""
    g = golden("acoustic_loop.npz")
    NX, NY, Tn, _ = loop_case(g)
    p = ads.AcousticPropagatorParams(NX=NX, NY=NY, NSTEP=Tn, DELTAX=float(g["h"]),
                                     DELTAY=float(g["h"]), DELTAT=float(g["dt"]),
                                     NPOINTS_PML=int(g["npml"]), vp_ref=float(g["vp_ref"]),
                                     PropagatorKernel=1)
    src = ads.AcousticSource(g["srci"], g["srcj"], g["srcv"])
    rcv = ads.AcousticReceiver(g["rcvi"], g["rcvj"])
    tr = ads.compute_forward_GPU(p, [src, src], [rcv, rcv], g["vp"])
    assert len(tr) == 2 and tuple(tr[0].shape) == g["rcvv"].shape
    assert rel(tr[0].cpu().numpy(), g["rcvv"]) <= TOL64 and torch.equal(tr[0], tr[1])


def test_one_shot_entry_points_match_the_golden(ads, cuda):
    """ads_acoustic_forward / ads_acoustic_gradient (plan, run, destroy in one
    call) on the reference's golden loop: bitwise the plan's own results."""
    import ctypes

    g = golden("acoustic_loop.npz")
    NX, NY, Tn, shot = loop_case(g)
    h, dt = float(g["h"]), float(g["dt"])
    plan = ads.AcousticPlan(NX, NY, h, h, dt, [shot], npml=int(g["npml"]),
                            vp_ref=float(g["vp_ref"]), precision="f64")
    vp = T(g["vp"].reshape(NX + 2, NY + 2), cuda)
    obs = T(g["obs"].reshape(-1), cuda)
    tr = plan.forward(vp)
    loss, grad = plan.gradient(vp, obs)
    L = ads.lib()
    st = ctypes.c_void_p(torch.cuda.current_stream().cuda_stream)
    tr1 = torch.empty_like(tr)
    ads._lib.check(L.ads_acoustic_forward(ctypes.byref(plan._cfg), plan._arr, vp.data_ptr(),
                                          tr1.data_ptr(), st))
    loss1 = torch.empty(1, dtype=torch.float64, device=cuda)
    grad1 = torch.empty_like(grad)
    ads._lib.check(L.ads_acoustic_gradient(ctypes.byref(plan._cfg), plan._arr, vp.data_ptr(),
                                           obs.data_ptr(), loss1.data_ptr(), grad1.data_ptr(),
                                           st))
    assert torch.equal(tr, tr1) and torch.equal(loss.reshape(1), loss1)
    assert torch.equal(grad, grad1)
    assert rel(tr1.cpu().numpy(), g["rcvv"].reshape(-1)) <= TOL64
    with pytest.raises(ads.AdsError):
        ads._lib.check(L.ads_acoustic_forward(None, plan._arr, vp.data_ptr(), tr1.data_ptr(), st))
    plan.close()


def test_fwi_lbfgs_reduces_misfit(ads, cuda):
    """The L-BFGS FWI loop on the batched FP32 gradient (4 shots): the misfit
    falls well below its starting value and the loss history is recorded."""
    pytest.importorskip("scipy")
    NX, NY, npml, NT, h, dt = 60, 50, 10, 400, 10.0, 1e-3
    vt = ads.layered_gaussian_model(NX + 2, NY + 2, 2000.0, 3000.0, seed=5)
    v0 = ads.gaussian_smooth(vt, sigma=4.0)
    p = ads.AcousticPropagatorParams(NX=NX, NY=NY, NSTEP=NT, DELTAT=dt)
    wav = ads.Ricker(p, ads.ricker_width_samples(15.0, dt), 1.5 / 15.0 / dt, 1e6)
    shots = [dict(x0=0, nx=NX, nstep=NT, srci=[si], srcj=[npml + 4], srcv=wav[:, None],
                  rcvi=np.arange(npml + 2, NX - npml), rcvj=np.full(NX - 2 * npml - 2, npml + 3))
             for si in (15, 25, 35, 45)]
    plan = ads.AcousticPlan(NX, NY, h, h, dt, shots, npml=npml, vp_ref=2500.0, precision="f32")
    obs = plan.forward(T(vt, cuda)).clone()
    l0 = float(plan.gradient(T(v0, cuda), obs)[0])
    seen = []
    vp, losses = ads.fwi_lbfgs(plan, v0, obs, max_iter=8,
                               callback=lambda x, it, loss: seen.append(it),
                               vmin=1500.0, vmax=3500.0)
    assert len(losses) == len(seen) >= 4
    assert losses[-1] < 0.5 * l0, (l0, losses)
    assert np.all(vp >= 1500.0 - 1e-9) and np.all(vp <= 3500.0 + 1e-9)
    plan.close()


@pytest.mark.parametrize("resident", [-1, 2])
def test_tma_interior_forward_is_bitwise_the_register_kernel(ads, cuda, resident):
    """FP32 plans with tma = 1 step their interior items through tensor-map
    tile copies (k_ac_fwd_tma); the arithmetic is the register-queue kernel's,
    so traces, loss and gradient are bitwise those of the default plan.
    Uneven shots, odd checkpoint spacing and resident segments exercise the
    ring (MODE 0, with checkpoints), the recompute (MODE 1) and the resident
    store (MODE 2)."""
    rng = np.random.default_rng(17)
    MX, MY, npml = 360, 300, 20
    shots = []
    for k, (x0, nx, T) in enumerate([(0, 360, 70), (40, 250, 55), (100, 197, 64)]):
        nr = 40
        shots.append(dict(x0=x0, nx=nx, nstep=T, srci=[nx // 2 + k], srcj=[npml + 8],
                          srcv=rng.standard_normal((T, 1)),
                          rcvi=np.linspace(2, nx - 1, nr).astype(int), rcvj=np.full(nr, npml + 3)))
    vp = torch.as_tensor(2000 + 800 * rng.random((MX + 2, MY + 2)), device="cuda")
    out = {}
    for tma in (1, 0):
        plan = ads.AcousticPlan(MX, MY, 10.0, 10.0, 1e-3, shots, npml=npml, vp_ref=2400.0,
                                precision="f32", ckpt_every=9, resident_segments=resident,
                                rows_per_thread=4, tma=tma)
        assert plan.uses_tma == (tma == 1)
        obs = plan.forward(vp * 1.02).clone()
        tr = plan.forward(vp).clone()
        loss, grad = plan.gradient(vp, obs)
        torch.cuda.synchronize()
        plan.device_status()
        out[tma] = (tr.cpu(), float(loss), grad.cpu())
        plan.close()
    assert torch.equal(out[1][0], out[0][0])
    assert out[1][1] == out[0][1]
    assert torch.equal(out[1][2], out[0][2])
