"""ScatterAddOps / GatherOps / AddSource / GetReceive through the C ABI against
the reference's compiled CPU operators (golden fixtures)."""
import ctypes as C

import numpy as np
import pytest
import torch

from conftest import golden

pytestmark = pytest.mark.gpu


def P(t):
    return C.c_void_p(t.data_ptr()) if t is not None else None


def S():
    return C.c_void_p(torch.cuda.current_stream().cuda_stream)


def test_add_source_and_grad(ads, cuda):
    from adseismic_gb300._lib import call

    g = golden("index_ops.npz")
    NX, NY = int(g["NX"]), int(g["NY"])
    N = (NX + 2) * (NY + 2)
    in5 = torch.tensor(g["in5"], device=cuda).view(5, N)
    # AddSource field order is (sxx, syy, sxy, vx, vy); the fixture holds (vx, vy, sxx, syy, sxy)
    order = [2, 3, 4, 0, 1]
    ins = [in5[k].contiguous() for k in order]
    outs = [torch.empty(N, dtype=torch.float64, device=cuda) for _ in range(5)]
    idx = [torch.tensor(g[k], device=cuda) for k in ("srci", "srcj", "srctype")]
    sv = torch.tensor(g["srcv"], device=cuda)
    call("ads_add_source_f64", *[P(t) for t in outs], *[P(t) for t in ins], *[P(t) for t in idx],
         len(g["srci"]), NX, NY, P(sv), S())
    got = torch.stack([outs[order.index(k)] for k in range(5)]).cpu().numpy().reshape(-1)
    assert np.array_equal(got, g["out5"])
    # in place
    call("ads_add_source_f64", *[P(t) for t in ins], *[P(t) for t in ins], *[P(t) for t in idx],
         len(g["srci"]), NX, NY, P(sv), S())
    got = torch.stack([ins[order.index(k)] for k in range(5)]).cpu().numpy().reshape(-1)
    assert np.array_equal(got, g["out5"])
    g5 = torch.tensor(g["g5"], device=cuda).view(5, N)
    gouts = [g5[k].contiguous() for k in order]
    gins = [torch.empty(N, dtype=torch.float64, device=cuda) for _ in range(5)]
    gs = torch.empty(len(g["srci"]), dtype=torch.float64, device=cuda)
    call("ads_add_source_bwd_f64", *[P(t) for t in gins], P(gs), *[P(t) for t in gouts],
         *[P(t) for t in idx], len(g["srci"]), NX, NY, S())
    got = torch.stack([gins[order.index(k)] for k in range(5)]).cpu().numpy().reshape(-1)
    assert np.array_equal(got, g["gin5"])
    assert np.array_equal(gs.cpu().numpy(), g["grad_srcv"])


def test_get_receive_and_grad(ads, cuda):
    from adseismic_gb300._lib import call

    g = golden("index_ops.npz")
    NX, NY, nt = int(g["NX"]), int(g["NY"]), int(g["nt"])
    f5 = [torch.tensor(g["f5"][k], device=cuda).contiguous() for k in range(5)]
    idx = [torch.tensor(g[k], device=cuda) for k in ("rcvi", "rcvj", "rcvtype")]
    nr = len(g["rcvi"])
    out = torch.empty(nr * nt, dtype=torch.float64, device=cuda)
    call("ads_get_receive_f64", P(out), *[P(t) for t in f5], nt, *[P(t) for t in idx], nr, NX,
         NY, S())
    assert np.array_equal(out.cpu().numpy().reshape(nr, nt), g["rec"])
    gf = [torch.empty_like(f5[0]) for _ in range(5)]
    gout = torch.tensor(g["gout"], device=cuda)
    call("ads_get_receive_bwd_f64", *[P(t) for t in gf], P(gout), nt, *[P(t) for t in idx], nr,
         NX, NY, S())
    for a, b in zip(gf, g["grec"]):
        assert np.allclose(a.cpu().numpy(), b, rtol=0, atol=1e-15)


def test_scatter_add_and_gather(ads, orc, cuda):
    from adseismic_gb300._lib import call

    rng = np.random.default_rng(1)
    d, n = 500, 40
    ipt = rng.standard_normal(d)
    ii = rng.choice(np.arange(1, d + 1), n, replace=False)
    upd = rng.standard_normal(n)
    ref = ipt.copy()
    for k in range(n):
        ref[ii[k] - 1] += upd[k]
    ti, tu, tp = (torch.tensor(x, device=cuda) for x in (ii, upd, ipt))
    out = torch.empty_like(tp)
    call("ads_scatter_add_f64", P(out), P(tp), P(ti), P(tu), d, n, S())
    assert np.array_equal(out.cpu().numpy(), ref)
    gout = torch.empty(n, dtype=torch.float64, device=cuda)
    call("ads_gather_f64", P(gout), P(tp), P(ti), n, S())
    assert np.array_equal(gout.cpu().numpy(), ipt[ii - 1])


def test_bad_indices_are_skipped_and_flagged(ads, cuda):
    from adseismic_gb300._lib import call

    d = 10
    tp = torch.zeros(d, dtype=torch.float64, device=cuda)
    ti = torch.tensor([0, 3, 11], device=cuda)
    tu = torch.ones(3, dtype=torch.float64, device=cuda)
    flags = C.c_int(0)
    call("ads_device_index_errors", 1, C.byref(flags))
    call("ads_scatter_add_f64", P(tp), P(tp), P(ti), P(tu), d, 3, S())
    call("ads_device_index_errors", 1, C.byref(flags))
    assert flags.value & 1
    assert tp.cpu().numpy()[2] == 1.0 and tp.sum().item() == 1.0
