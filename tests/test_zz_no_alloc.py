"""The allocation-free elastic step transpose (ads_elastic_step_bwd_f64_noalloc).

It serves callers that cannot allocate device memory while the step runs (for
example an operator inside another framework's custom-call hook, where that
framework owns the device memory).  Its scratch is a fixed
array inside the library, shared by every call, so this test checks it against
the allocating entry point ads_elastic_step_bwd_f64 on two calls in a row with
different inputs: the second call must not see the first call's scratch.  The
file is named so that pytest collects it last."""
import ctypes as C

import numpy as np
import pytest
import torch

from conftest import golden

pytestmark = pytest.mark.gpu

TOL = 1e-13  # same kernels, same order: results agree to rounding (relative L2)


def rel(a, b):
    return np.linalg.norm(a - b) / max(np.linalg.norm(b), 1e-300)


def _call(name, ptrs, consts):
    from adseismic_gb300._lib import call

    call(name, *[C.c_void_p(p.data_ptr()) for p in ptrs], *consts,
         C.c_void_p(torch.cuda.current_stream().cuda_stream))


def _run(name, state, gout, lam, mu, rho, ax, bx, ay, by, dt, dx, dy, NX, NY):
    gin = torch.full_like(state, float("nan"))
    gl, gm, gr = (torch.zeros_like(lam) for _ in range(3))
    _call(name, [state, gout, gin, gl, gm, gr, lam, mu, rho, ax, bx, ay, by],
          [dt, dx, dy, NX, NY])
    torch.cuda.synchronize()
    return [t.cpu().numpy() for t in (gin, gl, gm, gr)]


def test_noalloc_matches_allocating_entry_point_on_two_calls(ads, cuda):
    g = golden("elastic_small.npz")
    NX, NY = int(g["NX"]), int(g["NY"])
    N = (NX + 2) * (NY + 2)
    dt, dx, dy = float(g["dt"]), float(g["dx"]), float(g["dy"])
    t = lambda a: torch.as_tensor(np.ascontiguousarray(a), dtype=torch.float64, device=cuda)
    model = [t(g["lam"]), t(g["mu"]), t(g["rho"])]
    prof = [t(g["ax"]), t(g["bx"]), t(g["ay"]), t(g["by"])]
    rng = np.random.default_rng(2024)
    for call_no in range(2):
        state = t(rng.standard_normal(13 * N) * (1 + call_no))
        gout = t(rng.standard_normal(13 * N))
        ref = _run("ads_elastic_step_bwd_f64", state, gout, *model, *prof, dt, dx, dy, NX, NY)
        got = _run("ads_elastic_step_bwd_f64_noalloc", state, gout, *model, *prof, dt, dx, dy,
                   NX, NY)
        for a, b in zip(got, ref):
            assert np.isfinite(a).all()
            assert rel(a, b) <= TOL, call_no


def test_noalloc_rejects_grids_beyond_its_scratch(ads, cuda):
    from adseismic_gb300._lib import ADS_ERR_INVALID, lib

    x = torch.zeros(16, dtype=torch.float64, device=cuda)
    p = C.c_void_p(x.data_ptr())
    rc = lib().ads_elastic_step_bwd_f64_noalloc(*([p] * 13), 1e-3, 10.0, 10.0, 300, 300,
                                                None)
    assert rc == ADS_ERR_INVALID
    assert "exceeds" in lib().ads_last_error().decode()
