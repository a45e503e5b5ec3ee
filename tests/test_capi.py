"""The C-ABI library loads and exports every symbol include/*.h declares; the
host-only helpers agree with the oracle.  No device compute is called here."""
import ctypes
import glob
import os
import re

import numpy as np
import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def declared_functions():
    names = set()
    for h in glob.glob(os.path.join(ROOT, "include", "*.h")):
        src = open(h).read()
        src = re.sub(r"/\*.*?\*/", "", src, flags=re.S)
        for m in re.finditer(r"^\s*(?:const\s+)?[A-Za-z_][\w\s\*]*?\b(ads_\w+)\s*\(", src,
                             re.M):
            names.add(m.group(1))
    return sorted(names)


def test_header_declares_entry_points():
    names = declared_functions()
    for n in ("ads_acoustic_step_fwd_f64", "ads_acoustic_step_bwd_f64", "ads_add_source_f64",
              "ads_get_receive_f64", "ads_elastic_step_fwd_f64", "ads_acoustic_plan_gradient",
              "ads_elastic_plan_gradient"):
        assert n in names


def test_library_exports_every_declared_symbol(ads):
    lib = ctypes.CDLL(ads.LIB_PATH)
    missing = [n for n in declared_functions() if not hasattr(lib, n)]
    assert not missing, missing


def test_python_binding_covers_the_header(ads):
    from adseismic_gb300 import _lib

    assert set(declared_functions()) <= set(_lib.EXPORTED)


def test_pml_profiles_match_oracle(ads, orc):
    NX, NY = 40, 30
    p = ads.AcousticPropagatorParams(NX=NX, NY=NY, DELTAX=10.0, DELTAY=12.0, NPOINTS_PML=7,
                                     vp_ref=1800.0)
    Sx, Sy = ads.compute_acoustic_PML_Params(p)
    s, t = orc.acoustic_pml(NX, NY, 10.0, 12.0, 7, 1800.0)
    assert np.array_equal(Sx.reshape(-1), s) and np.array_equal(Sy.reshape(-1), t)
    assert p.damping_x == pytest.approx(1800.0 / 70.0 * np.log(1000.0), rel=1e-15)
    assert p.damping_y == pytest.approx(1800.0 / 84.0 * np.log(1000.0), rel=1e-15)
    assert Sx[0].max() == pytest.approx(p.damping_x, rel=1e-12)  # d = L at the edge


def test_cpml_profiles_match_oracle(ads, orc):
    p = ads.ElasticPropagatorParams(NX=50, NY=40, DELTAX=10.0, DELTAY=11.0, DELTAT=8e-4,
                                    NPOINTS_PML=9, vp_ref=3100.0, f0=7.0)
    got = ads.compute_elastic_PML_Params(p)
    ref = orc.elastic_cpml(50, 40, 10.0, 11.0, 8e-4, 9, 3100.0, 7.0)
    for a, b in zip(got, ref):
        assert np.allclose(a.reshape(-1), b, rtol=1e-15, atol=1e-300)


def test_invalid_arguments_are_rejected_without_launch(ads):
    from adseismic_gb300 import _lib

    L = _lib.lib()
    rc = L.ads_acoustic_pml_profiles(0, 5, 1.0, 1.0, 3, 1000.0, 0.001, 15, None, None)
    assert rc == _lib.ADS_ERR_INVALID
    assert "NX" in L.ads_last_error().decode()


def test_null_arguments_are_rejected_before_any_device_call(ads):
    """The plan and one-shot entry points check their handles and configs
    first, so these fail the same way with or without a GPU."""
    from adseismic_gb300 import _lib

    L = _lib.lib()
    calls = [
        L.ads_acoustic_forward(None, None, None, None, None),
        L.ads_acoustic_gradient(None, None, None, None, None, None, None),
        L.ads_elastic_forward(None, None, None, None, None, None, None),
        L.ads_elastic_gradient(*([None] * 11)),
        L.ads_acoustic_plan_set_source_values(None, 0, None, None),
        L.ads_elastic_plan_set_source_values(None, 0, None, None),
        L.ads_acoustic_plan_gradient_ex(*([None] * 8)),
        L.ads_elastic_plan_gradient_ex(*([None] * 12)),
    ]
    assert calls == [_lib.ADS_ERR_INVALID] * len(calls), calls
    assert L.ads_acoustic_plan_source_offset(None, 0) == -1
    assert L.ads_elastic_plan_source_offset(None, 0) == -1
    assert L.ads_elastic_plan_resident_segments(None) == -1
    assert all(L.ads_acoustic_plan_rows(None, w) == -1 for w in range(4))
    assert all(L.ads_elastic_plan_rows(None, w) == -1 for w in range(2, 6))
    assert L.ads_acoustic_plan_tma(None) == -1
    assert L.ads_acoustic_plan_steps_per_block(None) == -1


def test_compute_calls_fail_loudly_without_gpu(ads):
    import torch

    if torch.cuda.is_available():
        pytest.skip("a GPU is present")
    from adseismic_gb300 import _lib

    rc = _lib.lib().ads_acoustic_step_fwd_f64(*([None] * 7), 0.1, 0.1, 0.1, 4, 4, None, None,
                                             None, 0, None)
    assert rc == _lib.ADS_ERR_CUDA
    assert "no CUDA device" in _lib.lib().ads_last_error().decode()


def test_ctypes_structs_match_the_header_layout(ads, tmp_path):
    """Sizes and field offsets of the config / shot structs as the C compiler
    lays them out from include/adseismic_gb300.h, against the ctypes binding."""
    import shutil
    import subprocess

    from adseismic_gb300 import _lib

    if shutil.which("gcc") is None:
        pytest.skip("gcc not available")
    structs = {"ads_acoustic_config": _lib.AcousticConfig, "ads_acoustic_shot": _lib.AcousticShot,
               "ads_elastic_config": _lib.ElasticConfig, "ads_elastic_shot": _lib.ElasticShot}
    lines = ["#include <stddef.h>", "#include <stdio.h>", '#include "adseismic_gb300.h"',
             "int main(void) {"]
    for cname, cls in structs.items():
        lines.append(f'  printf("{cname} %zu\\n", sizeof({cname}));')
        for fname, _ in cls._fields_:
            lines.append(f'  printf("{cname}.{fname} %zu\\n", offsetof({cname}, {fname}));')
    lines += ["  return 0;", "}"]
    src = tmp_path / "layout.c"
    src.write_text("\n".join(lines))
    exe = tmp_path / "layout"
    subprocess.run(["gcc", "-std=c11", "-I", os.path.join(ROOT, "include"), str(src), "-o",
                    str(exe)], check=True)
    got = dict(l.split() for l in subprocess.run([str(exe)], check=True, capture_output=True,
                                                 text=True).stdout.splitlines())
    for cname, cls in structs.items():
        assert int(got[cname]) == ctypes.sizeof(cls), cname
        for fname, _ in cls._fields_:
            assert int(got[f"{cname}.{fname}"]) == getattr(cls, fname).offset, (cname, fname)


# ------------------------------------------------- column-major (Julia) callers
# A Julia Array holds element (i, j) of an (n, m) matrix at i + j n.  The Julia
# shims pass permutedims(A, (2, 1)) into the ABI and read an (n, m) row-major
# result v back as permutedims(reshape(v, m, n), (2, 1)).  These helpers emulate
# that memory on numpy arrays.

def julia_memory(A):
    """The memory of a Julia array with A's elements (column-major)."""
    return np.asfortranarray(A).ravel(order="K")


def to_abi(A):
    """Memory of permutedims(A, (2, 1)): A in the ABI's row-major order."""
    return julia_memory(np.ascontiguousarray(np.asarray(A).T))


def from_abi(v, n, m):
    """permutedims(reshape(v, m, n), (2, 1)): Julia reshape fills columns first."""
    return np.reshape(np.asarray(v), (m, n), order="F").T


def test_julia_layout_conversion_matches_the_abi_order(ads, orc):
    """A non-square model held column-major, converted as the shims do, gives the
    oracle's traces and gradient on the row-major model; passed unconverted it
    would not."""
    NX, NY, T, h, dt = 17, 9, 60, 10.0, 1e-3
    rng = np.random.default_rng(4)
    vp = 2000.0 + 500.0 * rng.random((NX + 2, NY + 2))     # the Julia (NX+2, NY+2) model
    vp_julia = np.asfortranarray(vp)
    abi = to_abi(vp_julia)
    assert np.array_equal(abi, vp.reshape(-1))               # i*(NY+2) + j order
    assert not np.array_equal(julia_memory(vp_julia), vp.reshape(-1))
    # the reference's own sigma_ij = constant(param.Σx'[:]) is the same conversion
    Sx, Sy = ads.compute_acoustic_PML_Params(
        ads.AcousticPropagatorParams(NX=NX, NY=NY, DELTAX=h, DELTAY=h, NPOINTS_PML=3))
    assert np.array_equal(julia_memory(Sx.T), to_abi(Sx))
    sx, ty = orc.acoustic_pml(NX, NY, h, h, 3, 1000.0)
    srcv = rng.standard_normal((T, 1))
    srci, srcj, rcvi, rcvj = [9], [5], np.arange(2, NX + 2), np.full(NX, 3)
    ref = orc.acoustic_forward(NX, NY, T, dt, h, h, sx, ty, vp.reshape(-1), srci, srcj, srcv,
                               rcvi, rcvj)
    got = orc.acoustic_forward(NX, NY, T, dt, h, h, sx, ty, abi, srci, srcj, srcv, rcvi, rcvj)
    # the (T+1, nrcv) row-major buffer read back as the Julia matrix rcv.rcvv
    assert np.array_equal(from_abi(got.reshape(-1), T + 1, NX), ref)
    bad = orc.acoustic_forward(NX, NY, T, dt, h, h, sx, ty, julia_memory(vp_julia), srci, srcj,
                               srcv, rcvi, rcvj)
    assert not np.allclose(bad, ref)
    obs = ref * 1.01
    _, gref = orc.acoustic_gradient(NX, NY, T, dt, h, h, sx, ty, vp.reshape(-1), srci, srcj,
                                    srcv, rcvi, rcvj, obs)
    _, g = orc.acoustic_gradient(NX, NY, T, dt, h, h, sx, ty, abi, srci, srcj, srcv, rcvi,
                                 rcvj, to_abi(obs))
    assert np.array_equal(from_abi(g, NX + 2, NY + 2), gref.reshape(NX + 2, NY + 2))
