"""MAT model / source / receiver loaders (src/IO.jl:4-161).

Same file layout and semantics as the reference:
- scalars nx, ny (padded sizes, so NX = nx - 2, NY = ny - 2), nt, dx, dy, dt (and f0 for
  elastic models);
- the model arrays vp (and vs, rho for elastic) of shape (nx, ny);
- a `source` struct array with fields ix, iy (1-based, padded grid), vec ((nt, nsrc) or
  its transpose) and, for elastic sources, type;
- a `receiver` struct array with fields ix, iy (and type).

MAT v5 files are read with scipy.io; MAT v7.3 (HDF5) files need h5py, which is not a
dependency, and are rejected with a clear error.
"""
from __future__ import annotations

from dataclasses import dataclass

import numpy as np

from .acoustic import (AcousticPropagatorParams, AcousticPropagatorSolver, AcousticReceiver,
                       AcousticSource)
from .elastic import (ElasticPropagatorParams, ElasticPropagatorSolver, ElasticReceiver,
                      ElasticSource)
from .utils import compute_properties


def _matread(filename):
    from scipy.io import loadmat

    with open(filename, "rb") as f:
        head = f.read(128)
    if head.startswith(b"version https://git-lfs"):
        raise ValueError(f"{filename} is a git-lfs pointer, not MAT data")
    if b"MATLAB 7.3" in head:
        raise ValueError(f"{filename} is MAT v7.3 (HDF5): h5py is needed to read it")
    return loadmat(filename, squeeze_me=True, struct_as_record=False)


def _scalar(x):
    return np.asarray(x).reshape(-1)[0].item()


def _vec(x, dtype):
    """safe_vec: a scalar or an array as a 1-D array."""
    return np.atleast_1d(np.asarray(x, dtype=dtype)).reshape(-1)


def _structs(x):
    if isinstance(x, np.ndarray):
        return list(x.reshape(-1))
    return [x]


def _source_matrix(vec, nt):
    """src.vec as (nt, nsrc) (src/IO.jl:78-83, :151-154)."""
    v = np.asarray(vec, dtype=np.float64)
    if v.ndim == 1:
        v = v.reshape(-1, 1)
    if v.shape[0] != nt and v.shape[1] == nt:
        v = v.T
    if v.shape[0] == 1 and nt != 1:
        v = v.reshape(-1, 1)
    if v.shape[0] != nt:
        raise ValueError(f"source wavelet has {v.shape[0]} samples, the model nt = {nt}")
    return np.ascontiguousarray(v)


def load_params(filename, option="Acoustic", **kwargs):
    """src/IO.jl:4-25 (Acoustic / Elastic)."""
    d = _matread(filename)
    common = dict(NX=int(_scalar(d["nx"])) - 2, NY=int(_scalar(d["ny"])) - 2,
                  NSTEP=int(_scalar(d["nt"])), DELTAX=float(_scalar(d["dx"])),
                  DELTAY=float(_scalar(d["dy"])), DELTAT=float(_scalar(d["dt"])))
    common.update(kwargs)
    if option == "Acoustic":
        return AcousticPropagatorParams(**common)
    if option == "Elastic":
        return ElasticPropagatorParams(**common)
    raise ValueError("option should be either Acoustic or Elastic")


@dataclass
class LoadedAcousticModel:
    """What load_acoustic_model returns: the parameters, the model, and (called
    with a source) the AcousticPropagatorSolver closure of src/IO.jl:119-129."""
    param: AcousticPropagatorParams
    vp: np.ndarray

    def __call__(self, src, precision="f64"):
        return AcousticPropagatorSolver(self.param, src, self.vp, precision=precision)


def load_acoustic_model(filename, inv_vp=False, vp=None, mask=None, **kwargs):
    """src/IO.jl:97-130.  inv_vp / mask mark the reference's TF variable as
    trainable; here the caller differentiates through the plans, so they are
    accepted and have no effect.  vp overrides the file's model."""
    del inv_vp, mask
    d = _matread(filename)
    param = load_params(filename, "Acoustic", **kwargs)
    model = np.asarray(d["vp"] if vp is None else vp, dtype=np.float64)
    if model.shape != (param.NX + 2, param.NY + 2):
        raise ValueError(f"vp has shape {model.shape}, expected {(param.NX + 2, param.NY + 2)}")
    return LoadedAcousticModel(param, model)


def load_acoustic_source(filename):
    """src/IO.jl:146-161: one AcousticSource per struct of `source`."""
    d = _matread(filename)
    nt = int(_scalar(d["nt"]))
    out = []
    for s in _structs(d["source"]):
        out.append(AcousticSource(_vec(s.ix, np.int64), _vec(s.iy, np.int64),
                                  _source_matrix(s.vec, nt)))
    return out


def load_acoustic_receiver(filename):
    """src/IO.jl:133-144: one AcousticReceiver per struct of `receiver`."""
    d = _matread(filename)
    if "receiver" not in d or np.size(d["receiver"]) == 0:
        return []
    return [AcousticReceiver(_vec(r.ix, np.int64), _vec(r.iy, np.int64))
            for r in _structs(d["receiver"])]


@dataclass
class LoadedElasticModel:
    """What load_elastic_model returns (src/IO.jl:27-40): parameters with
    vp_ref = mean(vp) and f0 = file f0 / 2, the Lame parameters and density,
    and (called with a source) the ElasticPropagatorSolver closure."""
    param: ElasticPropagatorParams
    lam: np.ndarray
    mu: np.ndarray
    rho: np.ndarray

    def __call__(self, src, precision="f64"):
        return ElasticPropagatorSolver(self.param, src, self.rho, self.lam, self.mu,
                                       precision=precision)


def load_elastic_model(filename, inv_vp=False, inv_vs=False, inv_rho=False, **kwargs):
    del inv_vp, inv_vs, inv_rho
    d = _matread(filename)
    vp = np.asarray(d["vp"], dtype=np.float64)
    kw = dict(vp_ref=float(vp.mean()), f0=float(_scalar(d["f0"])) / 2)
    kw.update(kwargs)
    param = load_params(filename, "Elastic", **kw)
    lam, mu, rho = compute_properties(vp, np.asarray(d["vs"], dtype=np.float64),
                                      np.asarray(d["rho"], dtype=np.float64))
    return LoadedElasticModel(param, lam, mu, rho)


def load_elastic_source(filename):
    """src/IO.jl:66-94: ix, iy, type, vec (nt, nsrc)."""
    d = _matread(filename)
    nt = int(_scalar(d["nt"]))
    return [ElasticSource(_vec(s.ix, np.int64), _vec(s.iy, np.int64), _vec(s.type, np.int64),
                          _source_matrix(s.vec, nt))
            for s in _structs(d["source"])]


def load_elastic_receiver(filename):
    """src/IO.jl:43-63: ix, iy, type."""
    d = _matread(filename)
    if "receiver" not in d or np.size(d["receiver"]) == 0:
        return []
    return [ElasticReceiver(_vec(r.ix, np.int64), _vec(r.iy, np.int64), _vec(r.type, np.int64))
            for r in _structs(d["receiver"])]
