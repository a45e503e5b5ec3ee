"""MAT loaders (src/IO.jl layout): synthetic round trips, and the reference's
own BP model file where the reference checkout is present (CPU only)."""
import os

import numpy as np
import pytest

sio = pytest.importorskip("scipy.io")


@pytest.fixture(scope="module")
def ads():
    import __graft_entry__ as g

    return g.load_package()


def _acoustic_file(path, nshots=3, nt=120, transpose=False):
    rng = np.random.default_rng(1)
    nx, ny = 42, 30
    srcs = np.empty((1, nshots), dtype=object)
    rcvs = np.empty((1, nshots), dtype=object)
    for k in range(nshots):
        vec = rng.standard_normal(nt if k == 0 else (nt, 2))
        if transpose and k:
            vec = vec.T
        srcs[0, k] = {"ix": np.array(10 + k) if k == 0 else np.array([10 + k, 12]),
                      "iy": np.array(5) if k == 0 else np.array([5, 6]), "vec": vec}
        rcvs[0, k] = {"ix": np.arange(3, 40), "iy": np.full(37, 4)}
    sio.savemat(path, {"vp": 2000 + rng.random((nx, ny)), "nx": nx, "ny": ny, "nt": nt,
                       "dx": 10.0, "dy": 12.5, "dt": 1e-3, "f0": 10, "source": srcs,
                       "receiver": rcvs})
    return nx, ny, nt


@pytest.mark.parametrize("transpose", [False, True])
def test_acoustic_mat_round_trip(ads, tmp_path, transpose):
    f = str(tmp_path / "m.mat")
    nx, ny, nt = _acoustic_file(f, transpose=transpose)
    m = ads.load_acoustic_model(f, inv_vp=True, NPOINTS_PML=8)
    assert (m.param.NX, m.param.NY, m.param.NSTEP) == (nx - 2, ny - 2, nt)
    assert (m.param.DELTAX, m.param.DELTAY, m.param.DELTAT) == (10.0, 12.5, 1e-3)
    assert m.param.NPOINTS_PML == 8 and m.vp.shape == (nx, ny)
    srcs = ads.load_acoustic_source(f)
    rcvs = ads.load_acoustic_receiver(f)
    assert len(srcs) == 3 and len(rcvs) == 3
    assert srcs[0].srcv.shape == (nt, 1) and list(srcs[0].srci) == [10]
    assert srcs[2].srcv.shape == (nt, 2) and list(srcs[2].srcj) == [5, 6]
    assert list(rcvs[1].rcvi) == list(range(3, 40))
    ap = m(srcs[0])
    assert ap.param is m.param


def test_elastic_mat_round_trip(ads, tmp_path):
    rng = np.random.default_rng(2)
    nx, ny, nt = 34, 26, 80
    vp = 3000 + 100 * rng.random((nx, ny))
    vs, rho = vp / 1.8, 2000 + rng.random((nx, ny))
    src = np.empty((1, 1), dtype=object)
    src[0, 0] = {"ix": np.array([10, 10]), "iy": np.array([8, 8]), "type": np.array([2, 3]),
                 "vec": rng.standard_normal((2, nt))}
    rcv = np.empty((1, 1), dtype=object)
    rcv[0, 0] = {"ix": np.arange(4, 30), "iy": np.full(26, 5), "type": np.zeros(26)}
    f = str(tmp_path / "e.mat")
    sio.savemat(f, {"vp": vp, "vs": vs, "rho": rho, "nx": nx, "ny": ny, "nt": nt, "dx": 5.0,
                    "dy": 5.0, "dt": 5e-4, "f0": 12, "source": src, "receiver": rcv})
    m = ads.load_elastic_model(f)
    assert (m.param.NX, m.param.NY, m.param.NSTEP) == (nx - 2, ny - 2, nt)
    assert m.param.f0 == 6.0 and abs(m.param.vp_ref - vp.mean()) < 1e-9
    np.testing.assert_allclose(m.mu, rho * vs * vs)
    np.testing.assert_allclose(m.lam, rho * vp * vp - 2 * rho * vs * vs)
    s = ads.load_elastic_source(f)[0]
    r = ads.load_elastic_receiver(f)[0]
    assert s.srcv.shape == (nt, 2) and list(s.srctype) == [2, 3]
    assert list(r.rcvtype) == [0] * 26


def test_mat_v73_and_lfs_pointers_rejected(ads, tmp_path):
    f = tmp_path / "p.mat"
    f.write_bytes(b"version https://git-lfs.github.com/spec/v1\noid sha256:00\nsize 1\n")
    with pytest.raises(ValueError, match="git-lfs"):
        ads.load_acoustic_model(str(f))


REF_SRC = os.environ.get("ADS_REFERENCE_SRC", "")
BP = os.path.join(REF_SRC, "examples", "invert_velocity_model", "models",
                  "BP-model-smooth.mat")


@pytest.mark.skipif(not REF_SRC or not os.path.exists(BP),
                    reason="ADS_REFERENCE_SRC does not name a reference checkout")
def test_reference_bp_model_loads(ads):
    m = ads.load_acoustic_model(BP)
    srcs, rcvs = ads.load_acoustic_source(BP), ads.load_acoustic_receiver(BP)
    assert m.vp.shape == (m.param.NX + 2, m.param.NY + 2)
    assert len(srcs) == len(rcvs) == 8
    for s in srcs:
        assert s.srcv.shape == (m.param.NSTEP, len(s.srci))
        assert s.srci.min() >= 1 and s.srci.max() <= m.param.NX + 2
