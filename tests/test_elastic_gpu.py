"""Elastic parity on the GPU: single step and its transpose against the oracle,
whole-path FP64 traces/gradients (rel-L2 <= 1e-12) and FP32 against the FP64
oracle."""
import numpy as np
import pytest
import torch

from conftest import golden

pytestmark = pytest.mark.gpu


def rel(a, b):
    a, b = np.asarray(a, dtype=np.float64), np.asarray(b, dtype=np.float64)
    return np.linalg.norm(a - b) / max(np.linalg.norm(b), 1e-300)


def params(ads, g, T=None):
    return ads.ElasticPropagatorParams(NX=int(g["NX"]), NY=int(g["NY"]),
                                       NSTEP=int(T or g["NSTEP"]), DELTAX=float(g["dx"]),
                                       DELTAY=float(g["dy"]), DELTAT=float(g["dt"]),
                                       NPOINTS_PML=int(g["npml"]), vp_ref=float(g["vp_ref"]),
                                       f0=float(g["f0"]))


def test_step_forward_and_transpose_vs_oracle(ads, orc, cuda):
    g = golden("elastic_small.npz")
    p = params(ads, g)
    NX, NY = p.NX, p.NY
    N = (NX + 2) * (NY + 2)
    prof = ads.compute_elastic_PML_Params(p)
    ax, bx, kx, ay, by, ky = [a.reshape(-1) for a in prof]
    rng = np.random.default_rng(12)
    st = rng.standard_normal(13 * N)
    lam, mu, rho = g["lam"], g["mu"], g["rho"]
    srci, srcj, srct, srcv = [15, 3, 15], [10, 4, 10], [2, 0, 2], [1.5, -2.0, 0.25]
    ref = orc.elastic_step_fwd(st, lam, mu, rho, ax, bx, ay, by, p.DELTAT, p.DELTAX, p.DELTAY,
                               NX, NY, srci, srcj, srct, srcv)
    t = lambda a: torch.as_tensor(a, dtype=torch.float64, device=cuda)
    got = ads.elastic_one_step(p, t(rho), t(lam), t(mu), t(st).view(13, N), prof, srci, srcj,
                               srcv, srct)
    assert rel(got.cpu().numpy().reshape(-1), ref) <= 1e-14
    w = rng.standard_normal(13 * N)
    gin, gl, gm, gr = orc.elastic_step_bwd(st, w, lam, mu, rho, ax, bx, ay, by, p.DELTAT,
                                           p.DELTAX, p.DELTAY, NX, NY)
    Gin, Gl, Gm, Gr = ads.elastic_one_step_grad(p, t(rho), t(lam), t(mu), t(st).view(13, N),
                                                t(w).view(13, N), prof)
    assert rel(Gin.cpu().numpy().reshape(-1), gin) <= 1e-13
    for a, b in ((Gl, gl), (Gm, gm), (Gr, gr)):
        assert rel(a.cpu().numpy(), b) <= 1e-13


def test_step_fp32_forward_and_transpose_vs_fp64_oracle(ads, orc, cuda):
    """ads_elastic_step_fwd_f32 / _bwd_f32 against the FP64 oracle on the same
    FP32-rounded inputs: rel-L2 <= 1e-5 for the state, its transpose and the
    lambda / mu / rho gradients."""
    g = golden("elastic_small.npz")
    p = params(ads, g)
    NX, NY = p.NX, p.NY
    N = (NX + 2) * (NY + 2)
    r32 = lambda a: np.asarray(a, dtype=np.float32).astype(np.float64)
    prof = [r32(a) for a in ads.compute_elastic_PML_Params(p)]
    ax, bx, kx, ay, by, ky = [a.reshape(-1) for a in prof]
    rng = np.random.default_rng(21)
    st = r32(rng.standard_normal(13 * N))
    lam, mu, rho = r32(g["lam"]), r32(g["mu"]), r32(g["rho"])
    srci, srcj, srct, srcv = [15, 3, 15], [10, 4, 10], [2, 0, 2], r32([1.5, -2.0, 0.25])
    ref = orc.elastic_step_fwd(st, lam, mu, rho, ax, bx, ay, by, p.DELTAT, p.DELTAX, p.DELTAY,
                               NX, NY, srci, srcj, srct, srcv)
    t = lambda a: torch.as_tensor(np.asarray(a), dtype=torch.float32, device=cuda)
    got = ads.elastic_one_step(p, t(rho), t(lam), t(mu), t(st).view(13, N),
                               [t(a) for a in prof], srci, srcj, srcv, srct)
    assert got.dtype == torch.float32
    assert rel(got.double().cpu().numpy().reshape(-1), ref) <= 1e-5
    w = r32(rng.standard_normal(13 * N))
    gin, gl, gm, gr = orc.elastic_step_bwd(st, w, lam, mu, rho, ax, bx, ay, by, p.DELTAT,
                                           p.DELTAX, p.DELTAY, NX, NY)
    Gin, Gl, Gm, Gr = ads.elastic_one_step_grad(p, t(rho), t(lam), t(mu), t(st).view(13, N),
                                                t(w).view(13, N), [t(a) for a in prof])
    assert Gin.dtype == Gl.dtype == torch.float32
    assert rel(Gin.double().cpu().numpy().reshape(-1), gin) <= 1e-5
    for a, b in ((Gl, gl), (Gm, gm), (Gr, gr)):
        assert rel(a.double().cpu().numpy(), b) <= 1e-5


def shots_from(g):
    return [dict(srci=g["srci"], srcj=g["srcj"], srctype=g["srctype"], srcv=g["srcv"],
                 rcvi=g["rcvi"], rcvj=g["rcvj"], rcvtype=g["rcvtype"])]


@pytest.mark.parametrize("use_graph", [True, False])
@pytest.mark.parametrize("ckpt", [0, 1, 17])
@pytest.mark.parametrize("resident", [-1, 0, 2])
def test_plan_fp64_vs_oracle(ads, cuda, use_graph, ckpt, resident):
    """resident: checkpoint segments whose adjoint inputs stay on the device
    (-1 none: every segment recomputed; 0 as many as fit: all here; 2 the
    last two)."""
    g = golden("elastic_small.npz")
    p = params(ads, g)
    plan = ads.ElasticPlan(p, shots_from(g), precision="f64", use_graph=use_graph,
                           ckpt_every=ckpt, resident_segments=resident)
    K = min(ckpt, p.NSTEP) if ckpt else min(p.NSTEP, 100)
    nseg = -(-p.NSTEP // K)
    assert plan.resident_segments == {-1: 0, 0: nseg, 2: min(2, nseg)}[resident]
    t = lambda a: torch.as_tensor(a, dtype=torch.float64, device=cuda)
    tr = plan.forward(t(g["lam"]), t(g["mu"]), t(g["rho"]))
    assert rel(tr.cpu().numpy(), g["rcvv"].reshape(-1)) <= 1e-12
    loss, gl, gm, gr = plan.gradient(t(g["lam"]), t(g["mu"]), t(g["rho"]),
                                     t(g["obs"].reshape(-1)))
    torch.cuda.synchronize()
    assert abs(float(loss) - float(g["loss"])) <= 1e-12 * float(g["loss"])
    for a, k in ((gl, "grad_lambda"), (gm, "grad_mu"), (gr, "grad_rho")):
        assert rel(a.cpu().numpy(), g[k]) <= 1e-12, k
    plan.close()


@pytest.mark.parametrize("precision,tol", [("f64", 1e-12), ("f32", 1e-4)])
def test_autotuned_plan_vs_oracle(ads, cuda, precision, tol):
    """The autotuner picks the fused-step tile and adjoint strip heights; the
    results stay the oracle's."""
    g = golden("elastic_small.npz")
    p = params(ads, g)
    plan = ads.ElasticPlan(p, shots_from(g), precision=precision, ckpt_every=17, autotune=True)
    # adjoint tile heights (fused, FP32) or strip heights (three passes, FP64)
    assert plan.rows_per_warp in (6, 8, 12, 16, 20, 24, 32)
    assert plan.rows_per_tile in (12, 16, 20, 24)
    t = lambda a: torch.as_tensor(a, dtype=torch.float64, device=cuda)
    loss, gl, gm, gr = plan.gradient(t(g["lam"]), t(g["mu"]), t(g["rho"]),
                                     t(g["obs"].reshape(-1)))
    torch.cuda.synchronize()
    assert abs(float(loss) - float(g["loss"])) <= tol * float(g["loss"])
    for a, k in ((gl, "grad_lambda"), (gm, "grad_mu"), (gr, "grad_rho")):
        assert rel(a.cpu().numpy(), g[k]) <= tol, k
    plan.close()


def test_plan_fp32_vs_fp64_oracle(ads, cuda):
    g = golden("elastic_small.npz")
    p = params(ads, g)
    plan = ads.ElasticPlan(p, shots_from(g), precision="f32", ckpt_every=9)
    t = lambda a: torch.as_tensor(a, dtype=torch.float64, device=cuda)
    loss, gl, gm, gr, tr = plan.gradient(t(g["lam"]), t(g["mu"]), t(g["rho"]),
                                         torch.as_tensor(g["obs"].reshape(-1), device=cuda),
                                         want_traces=True)
    torch.cuda.synchronize()
    assert rel(tr.double().cpu().numpy(), g["rcvv"].reshape(-1)) <= 1e-5
    for a, k in ((gl, "grad_lambda"), (gm, "grad_mu"), (gr, "grad_rho")):
        assert rel(a.cpu().numpy(), g[k]) <= 1e-4, k
    plan.close()


def test_multishot_sum_and_julia_api(ads, orc, cuda):
    g = golden("elastic_small.npz")
    p = params(ads, g, T=35)
    NX, NY = p.NX, p.NY
    prof = ads.compute_elastic_PML_Params(p)
    ax, bx, kx, ay, by, ky = [a.reshape(-1) for a in prof]
    rng = np.random.default_rng(2)
    shots, obs = [], []
    for s in range(3):
        ns = s + 1
        sh = dict(srci=rng.integers(3, NX, ns), srcj=rng.integers(3, NY, ns),
                  srctype=rng.integers(0, 5, ns), srcv=rng.standard_normal((35, ns)) * 1e5,
                  rcvi=rng.integers(1, NX + 3, 7), rcvj=rng.integers(1, NY + 3, 7),
                  rcvtype=rng.integers(0, 5, 7))
        shots.append(sh)
        obs.append(rng.standard_normal((7, 36)) * 1e-3)
    ref_loss, RL, RM, RR = 0.0, 0, 0, 0
    for sh, o in zip(shots, obs):
        l, a, b, c = orc.elastic_gradient(NX, NY, 35, p.DELTAT, p.DELTAX, p.DELTAY, ax, bx, ay,
                                          by, g["lam"], g["mu"], g["rho"], sh["srci"],
                                          sh["srcj"], sh["srctype"], sh["srcv"], sh["rcvi"],
                                          sh["rcvj"], sh["rcvtype"], o)
        ref_loss += l
        RL, RM, RR = RL + a, RM + b, RR + c
    plan = ads.ElasticPlan(p, shots, precision="f64", ckpt_every=8)
    t = lambda a: torch.as_tensor(a, dtype=torch.float64, device=cuda)
    loss, gl, gm, gr = plan.gradient(t(g["lam"]), t(g["mu"]), t(g["rho"]),
                                     plan.pack([t(o) for o in obs]))
    torch.cuda.synchronize()
    assert abs(float(loss) - ref_loss) <= 1e-12 * ref_loss
    for a, b in ((gl, RL), (gm, RM), (gr, RR)):
        assert rel(a.cpu().numpy(), b) <= 1e-12
    plan.close()
    src = ads.ElasticSource(shots[0]["srci"], shots[0]["srcj"], shots[0]["srctype"],
                            shots[0]["srcv"])
    rcv = ads.ElasticReceiver(shots[0]["rcvi"], shots[0]["rcvj"], shots[0]["rcvtype"])
    ep = ads.ElasticPropagatorSolver(p, src, g["rho"], g["lam"], g["mu"])
    ads.ElasticSimulatedObservation(ep, rcv)
    ref = orc.elastic_forward(NX, NY, 35, p.DELTAT, p.DELTAX, p.DELTAY, ax, bx, ay, by,
                              g["lam"], g["mu"], g["rho"], shots[0]["srci"], shots[0]["srcj"],
                              shots[0]["srctype"], shots[0]["srcv"], shots[0]["rcvi"],
                              shots[0]["rcvj"], shots[0]["rcvtype"], keep_history=True)
    assert rel(rcv.rcvv.cpu().numpy(), ref[0]) <= 1e-12
    # the reference's wavefield histories on the propagator (src/Struct.jl:64-73)
    hist = ref[1]
    assert tuple(ep.vx.shape) == (36, NX + 2, NY + 2) and tuple(ep.mem.shape)[1] == 8
    for k, f in enumerate((ep.vx, ep.vy, ep.sigmaxx, ep.sigmayy, ep.sigmaxy)):
        assert rel(f.cpu().numpy(), hist[:, k]) <= 1e-12, k
    assert rel(ep.mem.cpu().numpy(), hist[:, 5:]) <= 1e-12


@pytest.mark.parametrize("rows_per_warp,resident", [(0, 3), (5, -1), (5, 0)])
def test_plan_strips_tiles_and_edge_sources_vs_oracle(ads, orc, cuda, rows_per_warp, resident):
    """Several column strips and row tiles, an odd checkpoint interval (the
    step buffers alternate, so checkpoints land on both parities) and sources
    on cells no stencil updates (padded ring, box edges), which keep their
    value between steps and accumulate the source."""
    NX, NY, T = 61, 131, 41
    p = ads.ElasticPropagatorParams(NX=NX, NY=NY, NSTEP=T, DELTAX=10.0, DELTAY=10.0,
                                    DELTAT=0.8e-3, NPOINTS_PML=9, vp_ref=3000.0, f0=15.0)
    prof = ads.compute_elastic_PML_Params(p)
    ax, bx, kx, ay, by, ky = [a.reshape(-1) for a in prof]
    rng = np.random.default_rng(7)
    vp = 3000 + 300 * rng.random((NX + 2, NY + 2))
    lam, mu, rho = ads.compute_properties(vp, vp / 1.8, 2000 + 200 * rng.random((NX + 2, NY + 2)))
    lam, mu, rho = (a.reshape(-1) for a in (lam, mu, rho))
    # 1-based padded-grid cells: ring corners and edges, box edges, interior
    srci = np.array([1, NX + 2, 2, NX + 1, 2, 30, 31, 17, NX + 1, 2])
    srcj = np.array([1, NY + 2, 2, 5, NY + 1, 1, 60, 90, NY + 1, 70])
    srct = np.array([0, 1, 2, 4, 3, 2, 0, 4, 0, 1])
    srcv = rng.standard_normal((T, len(srci))) * 1e3
    rcvi = rng.integers(1, NX + 3, 25)
    rcvj = rng.integers(1, NY + 3, 25)
    rcvi[:3], rcvj[:3] = srci[:3], srcj[:3]
    rcvt = rng.integers(0, 5, 25)
    rcvt[:3] = srct[:3]
    obs = rng.standard_normal((25, T + 1)) * 1e-3
    sh = dict(srci=srci, srcj=srcj, srctype=srct, srcv=srcv, rcvi=rcvi, rcvj=rcvj, rcvtype=rcvt)
    ref_tr = orc.elastic_forward(NX, NY, T, p.DELTAT, p.DELTAX, p.DELTAY, ax, bx, ay, by, lam, mu,
                                 rho, srci, srcj, srct, srcv, rcvi, rcvj, rcvt)
    ref = orc.elastic_gradient(NX, NY, T, p.DELTAT, p.DELTAX, p.DELTAY, ax, bx, ay, by, lam, mu,
                               rho, srci, srcj, srct, srcv, rcvi, rcvj, rcvt, obs)
    t = lambda a: torch.as_tensor(a, dtype=torch.float64, device=cuda)
    plan = ads.ElasticPlan(p, [sh], precision="f64", ckpt_every=7,
                           rows_per_warp=rows_per_warp, resident_segments=resident)
    tr = plan.forward(t(lam), t(mu), t(rho))
    assert rel(tr.cpu().numpy(), ref_tr.reshape(-1)) <= 1e-12
    loss, gl, gm, gr = plan.gradient(t(lam), t(mu), t(rho), t(obs.reshape(-1)))
    torch.cuda.synchronize()
    assert abs(float(loss) - ref[0]) <= 1e-12 * ref[0]
    for a, b in zip((gl, gm, gr), ref[1:]):
        assert rel(a.cpu().numpy(), b) <= 1e-12
    plan.close()
    p32 = ads.ElasticPlan(p, [sh], precision="f32", ckpt_every=7, rows_per_warp=rows_per_warp,
                          resident_segments=resident)
    loss32, gl32, gm32, gr32 = p32.gradient(t(lam), t(mu), t(rho),
                                            torch.as_tensor(obs.reshape(-1), device=cuda))
    torch.cuda.synchronize()
    assert abs(float(loss32) - ref[0]) <= 1e-4 * ref[0]
    for a, b in zip((gl32, gm32, gr32), ref[1:]):
        assert rel(a.cpu().numpy(), b) <= 1e-4
    p32.close()


@pytest.mark.parametrize("precision,tol", [("f64", 1e-12), ("f32", 1e-4)])
@pytest.mark.parametrize("resident", [-1, 2, 0])
def test_source_time_gradient_vs_oracle(ads, orc, cuda, precision, tol, resident):
    """d loss / d srcv of an elastic plan (two shots, sources of every field
    type, one on the first row its stencil updates, one of an ignored type)
    against the oracle; a source on the padded frame is rejected."""
    g = golden("elastic_small.npz")
    p = params(ads, g, T=41)
    NX, NY, T = p.NX, p.NY, p.NSTEP
    prof = ads.compute_elastic_PML_Params(p)
    ax, bx, kx, ay, by, ky = [a.reshape(-1) for a in prof]
    rng = np.random.default_rng(8)
    cases = [dict(srci=[10, 15, 8, 20, 12, 2, 9], srcj=[9, 12, 14, 7, 10, 5, 9],
                  srctype=[0, 1, 2, 3, 4, 2, 7]),
             dict(srci=[14], srcj=[11], srctype=[2])]
    shots, obs, want = [], [], []
    for c in cases:
        srcv = rng.standard_normal((T, len(c["srci"]))) * 1e2
        sh = dict(srci=np.array(c["srci"]), srcj=np.array(c["srcj"]),
                  srctype=np.array(c["srctype"]), srcv=srcv, rcvi=g["rcvi"], rcvj=g["rcvj"],
                  rcvtype=g["rcvtype"])
        o = g["obs"][:, :T + 1] * 0.5
        out = orc.elastic_gradient(NX, NY, T, p.DELTAT, p.DELTAX, p.DELTAY, ax, bx, ay, by,
                                   g["lam"], g["mu"], g["rho"], sh["srci"], sh["srcj"],
                                   sh["srctype"], srcv, sh["rcvi"], sh["rcvj"], sh["rcvtype"],
                                   o, want_src=True)
        shots.append(sh)
        obs.append(o)
        want.append(out[4])
    t = lambda a: torch.as_tensor(a, dtype=torch.float64, device=cuda)
    plan = ads.ElasticPlan(p, shots, precision=precision, ckpt_every=9,
                           resident_segments=resident, source_gradient=True)
    dtype = torch.float64 if precision == "f64" else torch.float32
    packed = torch.cat([torch.as_tensor(o.reshape(-1), dtype=dtype, device=cuda) for o in obs])
    out = plan.gradient(t(g["lam"]), t(g["mu"]), t(g["rho"]), packed, want_source_grad=True)
    torch.cuda.synchronize()
    got = out[-1]
    for k in range(len(cases)):
        gk = got[k].cpu().numpy()
        assert gk.shape == want[k].shape
        assert rel(gk, want[k]) <= tol, (k, rel(gk, want[k]))
    assert np.all(got[0].cpu().numpy()[:, -1] == 0.0)  # the ignored type
    plan.close()
    p2 = ads.ElasticPlan(p, shots, precision=precision, ckpt_every=9)
    with pytest.raises(ads.AdsError):
        p2.gradient(t(g["lam"]), t(g["mu"]), t(g["rho"]), packed, want_source_grad=True)
    p2.close()
    frame = dict(shots[1], srci=np.array([1]))  # sxx on row 0: read, never updated
    with pytest.raises(ads.AdsError, match="padded frame"):
        ads.ElasticPlan(p, [frame], precision=precision, ckpt_every=9, source_gradient=True)


@pytest.mark.parametrize("precision", ["f64", "f32"])
def test_set_source_values_matches_a_fresh_plan(ads, cuda, precision):
    """Wavelets replaced in place (a source on the padded frame, which is
    added to both state buffers; an ignored type; a shot without sources)
    give bitwise the traces, loss and gradients of a plan created with them."""
    g = golden("elastic_small.npz")
    p = params(ads, g, T=40)
    rng = np.random.default_rng(9)
    base = dict(rcvi=g["rcvi"], rcvj=g["rcvj"], rcvtype=g["rcvtype"])
    shots = [dict(base, srci=g["srci"], srcj=g["srcj"], srctype=g["srctype"],
                  srcv=rng.standard_normal((40, len(g["srci"]))) * 1e2),
             dict(base, srci=[1, 14, 9], srcj=[5, 11, 9], srctype=[2, 4, 7],
                  srcv=rng.standard_normal((40, 3)) * 1e2),
             dict(base, srci=[], srcj=[], srctype=[], srcv=np.zeros((40, 0)))]
    zeroed = [dict(s, srcv=np.zeros_like(s["srcv"])) for s in shots]
    a = ads.ElasticPlan(p, shots, precision=precision, ckpt_every=9)
    b = ads.ElasticPlan(p, zeroed, precision=precision, ckpt_every=9)
    for k, s in enumerate(shots):
        b.set_source_values(k, torch.as_tensor(s["srcv"], dtype=torch.float64, device=cuda))
    t = lambda x: torch.as_tensor(x, dtype=torch.float64, device=cuda)
    m = (t(g["lam"]), t(g["mu"]), t(g["rho"]))
    ta, tb = a.forward(*m), b.forward(*m)
    assert torch.equal(ta, tb)
    ra, rb = a.gradient(*m, ta * 0.9), b.gradient(*m, ta * 0.9)
    torch.cuda.synchronize()
    assert all(torch.equal(x, y) for x, y in zip(ra, rb))
    with pytest.raises(ads.AdsError):
        b.set_source_values(-1, t(shots[0]["srcv"]))
    a.close()
    b.close()


def test_julia_named_multishot_helpers(ads, cuda):
    """compute_forward_GPU and compute_loss_and_grads_GPU with elastic
    parameters (model = (rho, lambda, mu), src/Utils.jl:300-332,574-601)
    against the oracle's golden traces, loss and gradients."""
    g = golden("elastic_small.npz")
    p = params(ads, g)
    src = ads.ElasticSource(g["srci"], g["srcj"], g["srctype"], g["srcv"])
    rcv = ads.ElasticReceiver(g["rcvi"], g["rcvj"], g["rcvtype"])
    model = (g["rho"], g["lam"], g["mu"])
    tr = ads.compute_forward_GPU(p, [src, src], [rcv, rcv], model)
    assert len(tr) == 2 and tuple(tr[0].shape) == g["rcvv"].shape
    assert rel(tr[0].cpu().numpy(), g["rcvv"]) <= 1e-12 and torch.equal(tr[0], tr[1])
    loss, gl, gm, gr = ads.compute_loss_and_grads_GPU(p, [src], [rcv], [g["obs"]], model)
    assert abs(float(loss) - float(g["loss"])) <= 1e-12 * float(g["loss"])
    for a, k in ((gl, "grad_lambda"), (gm, "grad_mu"), (gr, "grad_rho")):
        assert rel(a.cpu().numpy(), g[k]) <= 1e-12, k


def test_one_shot_entry_points_match_the_plan(ads, cuda):
    """ads_elastic_forward / ads_elastic_gradient (plan, run, destroy in one
    call): bitwise the plan's own traces, loss and gradients."""
    import ctypes

    g = golden("elastic_small.npz")
    p = params(ads, g)
    plan = ads.ElasticPlan(p, shots_from(g), precision="f64", ckpt_every=17)
    t = lambda a: torch.as_tensor(a, dtype=torch.float64, device=cuda)
    lam, mu, rho, obs = t(g["lam"]), t(g["mu"]), t(g["rho"]), t(g["obs"].reshape(-1))
    tr = plan.forward(lam, mu, rho)
    loss, gl, gm, gr = plan.gradient(lam, mu, rho, obs)
    L = ads.lib()
    st = ctypes.c_void_p(torch.cuda.current_stream().cuda_stream)
    tr1 = torch.empty_like(tr)
    ads._lib.check(L.ads_elastic_forward(ctypes.byref(plan._cfg), plan._arr, lam.data_ptr(),
                                         mu.data_ptr(), rho.data_ptr(), tr1.data_ptr(), st))
    out = [torch.empty(1, dtype=torch.float64, device=cuda)] + [torch.empty_like(lam)
                                                                 for _ in range(3)]
    ads._lib.check(L.ads_elastic_gradient(ctypes.byref(plan._cfg), plan._arr, lam.data_ptr(),
                                          mu.data_ptr(), rho.data_ptr(), obs.data_ptr(),
                                          *[o.data_ptr() for o in out], st))
    assert torch.equal(tr, tr1) and torch.equal(loss.reshape(1), out[0])
    assert all(torch.equal(a, b) for a, b in zip((gl, gm, gr), out[1:]))
    assert rel(tr1.cpu().numpy(), g["rcvv"].reshape(-1)) <= 1e-12
    with pytest.raises(ads.AdsError):
        ads._lib.check(L.ads_elastic_forward(ctypes.byref(plan._cfg), None, lam.data_ptr(),
                                             mu.data_ptr(), rho.data_ptr(), tr1.data_ptr(), st))
    plan.close()


@pytest.mark.parametrize("precision", ["f64", "f32"])
def test_fused_adjoint_all_item_kinds_vs_oracle_and_three_passes(ads, orc, cuda, precision):
    """The fused adjoint step (the default) on a grid with warp items of all
    four kinds (CPML-free, x-CPML rows, y-CPML columns, both), two shots, an
    odd checkpoint interval and two resident segments: against the oracle
    (FP64 1e-12, FP32 1e-4) and against the three gather passes on the same
    plan geometry (FP64 1e-13, FP32 1e-5: the same terms, with the 1 / (24 h)
    factor of each gather applied to its 4-term sum instead of to each term)."""
    NX, NY, T = 150, 190, 33
    p = ads.ElasticPropagatorParams(NX=NX, NY=NY, NSTEP=T, DELTAX=10.0, DELTAY=12.0,
                                    DELTAT=0.8e-3, NPOINTS_PML=10, vp_ref=3000.0, f0=15.0)
    prof = ads.compute_elastic_PML_Params(p)
    ax, bx, kx, ay, by, ky = [a.reshape(-1) for a in prof]
    rng = np.random.default_rng(31)
    vp = 3000 + 400 * rng.random((NX + 2, NY + 2))
    lam, mu, rho = ads.compute_properties(vp, vp / 1.7,
                                          2000 + 300 * rng.random((NX + 2, NY + 2)))
    lam, mu, rho = (a.reshape(-1) for a in (lam, mu, rho))
    shots, refs = [], []
    for k in range(2):
        srci = np.array([40 + 60 * k, 40 + 60 * k, 8, 75])
        srcj = np.array([95, 95, 120 - 50 * k, 6])
        srct = np.array([2, 3, 0, 4])
        srcv = rng.standard_normal((T, 4)) * 1e3
        nr = 60
        rcvi = rng.integers(2, NX, nr)
        rcvj = rng.integers(2, NY, nr)
        rcvt = rng.integers(0, 5, nr)
        obs = rng.standard_normal((nr, T + 1)) * 1e-3
        shots.append(dict(srci=srci, srcj=srcj, srctype=srct, srcv=srcv, rcvi=rcvi, rcvj=rcvj,
                          rcvtype=rcvt, obs=obs))
        if precision == "f64":
            refs.append(orc.elastic_gradient(NX, NY, T, p.DELTAT, p.DELTAX, p.DELTAY, ax, bx,
                                             ay, by, lam, mu, rho, srci, srcj, srct, srcv,
                                             rcvi, rcvj, rcvt, obs))
    obs = np.concatenate([s["obs"].reshape(-1) for s in shots])
    dt = torch.float64 if precision == "f64" else torch.float32
    t = lambda a: torch.as_tensor(a, dtype=torch.float64, device=cuda)
    out = {}
    for passes in (1, 3):
        plan = ads.ElasticPlan(p, shots, precision=precision, ckpt_every=7, rows_per_warp=16,
                               resident_segments=2, adjoint_passes=passes)
        if passes == 1:
            assert all(n > 0 for n in plan.adjoint_items), plan.adjoint_items
        else:
            assert plan.adjoint_items == [0, 0, 0, 0]
        loss, gl, gm, gr = plan.gradient(t(lam), t(mu), t(rho),
                                         torch.as_tensor(obs, dtype=dt, device=cuda))
        torch.cuda.synchronize()
        out[passes] = [float(loss)] + [a.cpu().numpy() for a in (gl, gm, gr)]
        plan.close()
    f, s3 = out[1], out[3]
    tol3 = 1e-13 if precision == "f64" else 1e-5
    assert abs(f[0] - s3[0]) <= tol3 * abs(s3[0])
    for a, b in zip(f[1:], s3[1:]):
        assert rel(a, b) <= tol3
    if precision == "f64":
        lref = sum(r[0] for r in refs)
        assert abs(f[0] - lref) <= 1e-12 * lref
        for k in range(3):
            assert rel(f[1 + k], sum(r[1 + k] for r in refs)) <= 1e-12


@pytest.mark.parametrize("use_graph", [True, False])
@pytest.mark.parametrize("resident", [-1, 2])
def test_fused_adjoint_fp64_golden_loop(ads, cuda, use_graph, resident):
    """The fused adjoint (adjoint_passes = 1) in an FP64 plan against the
    golden loop (rel-L2 <= 1e-12), with and without graphs, with every segment
    recomputed or the last two resident (the adjoint state alternates between
    two buffers, so odd and even segment lengths both occur)."""
    g = golden("elastic_small.npz")
    p = params(ads, g)
    plan = ads.ElasticPlan(p, shots_from(g), precision="f64", use_graph=use_graph,
                           ckpt_every=7, resident_segments=resident, adjoint_passes=1)
    assert all(n >= 0 for n in plan.adjoint_items) and sum(plan.adjoint_items) > 0
    t = lambda a: torch.as_tensor(a, dtype=torch.float64, device=cuda)
    loss, gl, gm, gr = plan.gradient(t(g["lam"]), t(g["mu"]), t(g["rho"]),
                                     t(g["obs"].reshape(-1)))
    torch.cuda.synchronize()
    assert abs(float(loss) - float(g["loss"])) <= 1e-12 * float(g["loss"])
    for a, k in ((gl, "grad_lambda"), (gm, "grad_mu"), (gr, "grad_rho")):
        assert rel(a.cpu().numpy(), g[k]) <= 1e-12, k
    plan.close()
