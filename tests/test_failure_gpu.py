"""Failure paths on the GPU, none of which faults the device.

- A plan larger than the device's memory is refused with ADS_ERR_NOMEM
  before any launch, and the library keeps working (acoustic and elastic).
- NaN in the model propagates to a NaN loss and gradient, and leaves no state
  behind: the next call on the same plan gives the clean result bit for bit.
- Non-finite or non-positive scalars are rejected with ADS_ERR_INVALID.
"""
import numpy as np
import pytest
import torch

pytestmark = pytest.mark.gpu

NOMEM, INVALID = 3, 1


def code_of(err):
    return int(str(err).split("(")[1].split(")")[0])


def small_acoustic(ads, precision="f64"):
    rng = np.random.default_rng(2)
    NX, NY, T = 30, 26, 40
    shot = dict(x0=0, nx=NX, nstep=T, srci=[12], srcj=[9], srcv=rng.standard_normal((T, 1)),
                rcvi=np.arange(3, 28), rcvj=np.full(25, 4))
    plan = ads.AcousticPlan(NX, NY, 10.0, 10.0, 1e-3, [shot], npml=5, vp_ref=2000.0,
                            precision=precision, ckpt_every=9)
    vp = torch.as_tensor(2000 + 300 * rng.random((NX + 2, NY + 2)), device="cuda")
    return plan, vp


def test_acoustic_plan_beyond_device_memory_is_refused(ads, cuda):
    # 400 shots of 1000 x 1000 in FP64: about 390 GB of wavefields and stores
    n = 400
    shots = [dict(x0=0, nx=1000, nstep=400, srci=[500], srcj=[50], srcv=np.ones((400, 1)),
                  rcvi=[10], rcvj=[10]) for _ in range(n)]
    free0 = torch.cuda.mem_get_info()[0]
    with pytest.raises(ads.AdsError) as e:
        ads.AcousticPlan(1000, 1000, 10.0, 10.0, 1e-3, shots, npml=20, precision="f64",
                         resident_segments=-1)
    assert code_of(e.value) == NOMEM and "GB" in str(e.value)
    assert torch.cuda.mem_get_info()[0] >= free0 - (1 << 28)  # nothing leaked
    plan, vp = small_acoustic(ads)  # the library still works
    obs = torch.zeros(plan.trace_count, dtype=torch.float64, device="cuda")
    loss, grad = plan.gradient(vp, obs)
    torch.cuda.synchronize()
    assert np.isfinite(float(loss)) and float(loss) > 0
    plan.close()


def test_elastic_plan_beyond_device_memory_is_refused(ads, cuda):
    p = ads.ElasticPropagatorParams(NX=1000, NY=1000, NSTEP=400, DELTAX=10.0, DELTAY=10.0,
                                    DELTAT=1e-3, NPOINTS_PML=20, vp_ref=3000.0, f0=10.0)
    shot = dict(srci=[500], srcj=[50], srctype=[2], srcv=np.ones((400, 1)), rcvi=[10],
                rcvj=[10], rcvtype=[0])
    with pytest.raises(ads.AdsError) as e:
        ads.ElasticPlan(p, [shot] * 300, precision="f64", resident_segments=-1)
    assert code_of(e.value) == NOMEM
    plan, vp = small_acoustic(ads)
    plan.forward(vp)
    torch.cuda.synchronize()
    plan.close()


@pytest.mark.parametrize("precision", ["f64", "f32"])
def test_nan_model_propagates_and_leaves_no_state(ads, cuda, precision):
    plan, vp = small_acoustic(ads, precision)
    obs = plan.forward(vp * 1.03).clone()
    l0, g0 = plan.gradient(vp, obs)
    l0, g0 = float(l0), g0.clone()
    bad = vp.clone()
    bad[15, 13] = float("nan")
    l1, g1 = plan.gradient(bad, obs)
    torch.cuda.synchronize()
    assert np.isnan(float(l1)) and torch.isnan(g1).any()
    l2, g2 = plan.gradient(vp, obs)
    torch.cuda.synchronize()
    assert float(l2) == l0 and torch.equal(g2, g0)
    plan.close()


@pytest.mark.parametrize("field,value", [("dt", float("nan")), ("dt", -1e-3), ("dx", 0.0),
                                         ("dx", float("inf"))])
def test_invalid_scalars_are_rejected(ads, cuda, field, value):
    kw = dict(dx=10.0, dt=1e-3)
    kw[field] = value
    shot = dict(x0=0, nx=20, nstep=10, srci=[5], srcj=[5], srcv=np.ones((10, 1)), rcvi=[3],
                rcvj=[3])
    with pytest.raises(ads.AdsError) as e:
        ads.AcousticPlan(20, 20, kw["dx"], 10.0, kw["dt"], [shot], npml=4)
    assert code_of(e.value) == INVALID
