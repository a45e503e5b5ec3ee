"""Write tests/golden/marmousi2_fwi.mat, the real-model fixture of the tests.

It is derived from the reference's examples/nn_fwi/models/marmousi2-model-smooth.mat
and marmousi2-model-true.mat (the Marmousi2 FWI example, src/IO.jl file
layout): the smooth file's scalars (nx, ny, nt, dx, dy, dt, f0), its model
arrays (vp, vs, rho, mask), its 8 sources and 8 receiver sets unchanged, plus
the true model's vp as `vp_true`, from which the tests simulate the observed
data.  MAT v5, compressed.  Run from the repository root, with
ADS_REFERENCE_SRC naming the reference checkout:

    ADS_REFERENCE_SRC=<checkout> python tests/golden/make_marmousi_fixture.py
"""
import os

import numpy as np
from scipy.io import loadmat, savemat

OUT = os.path.join(os.path.dirname(os.path.abspath(__file__)), "marmousi2_fwi.mat")


def _structs(arr, fields):
    arr = np.asarray(arr).reshape(-1)
    out = np.zeros((1, len(arr)), dtype=[(f, "O") for f in fields])
    for k, s in enumerate(arr):
        for f in fields:
            out[0, k][f] = np.asarray(s[f][0, 0])
    return out


def main():
    src = os.environ.get("ADS_REFERENCE_SRC", "")
    if not src or not os.path.isdir(src):
        raise SystemExit("set ADS_REFERENCE_SRC to the reference checkout")
    models = os.path.join(src, "examples", "nn_fwi", "models")
    smooth = loadmat(os.path.join(models, "marmousi2-model-smooth.mat"))
    true = loadmat(os.path.join(models, "marmousi2-model-true.mat"))
    d = {k: smooth[k] for k in ("nx", "ny", "nt", "dx", "dy", "dt", "f0", "vp", "vs", "rho",
                                "mask")}
    d["source"] = _structs(smooth["source"], ("ix", "iy", "vec"))
    d["receiver"] = _structs(smooth["receiver"], ("ix", "iy", "type"))
    d["vp_true"] = true["vp"]
    savemat(OUT, d, do_compression=True, format="5")
    print("wrote", OUT, os.path.getsize(OUT), "bytes")


if __name__ == "__main__":
    main()
