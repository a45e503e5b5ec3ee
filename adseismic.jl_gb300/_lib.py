"""ctypes binding of libadseismic_gb300.so (the C ABI in include/adseismic_gb300.h).

The library is the product: there is no Python or CPU fallback.  Loading fails
loudly when the shared object has not been built.
"""
from __future__ import annotations

import ctypes as C
import os

HERE = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(HERE, "lib", "libadseismic_gb300.so")

ADS_OK, ADS_ERR_INVALID, ADS_ERR_CUDA, ADS_ERR_NOMEM, ADS_ERR_UNSUPPORTED, ADS_ERR_TIMEOUT = range(6)
ADS_F64, ADS_F32 = 0, 1
ADS_VARIANT_W, ADS_VARIANT_U = 0, 1

_STATUS = {
    ADS_ERR_INVALID: "invalid argument",
    ADS_ERR_CUDA: "CUDA error",
    ADS_ERR_NOMEM: "out of device memory",
    ADS_ERR_UNSUPPORTED: "unsupported",
    ADS_ERR_TIMEOUT: "a bounded device wait ran out",
}


class AdsError(RuntimeError):
    """Raised when a C-ABI call returns a non-zero status."""

    def __init__(self, code: int, msg: str):
        super().__init__(f"{_STATUS.get(code, 'error')} ({code}): {msg}")
        self.code = code


class AcousticConfig(C.Structure):
    _fields_ = [
        ("MX", C.c_int64), ("MY", C.c_int64),
        ("dx", C.c_double), ("dy", C.c_double), ("dt", C.c_double),
        ("npml", C.c_int64), ("Rcoef", C.c_double), ("vp_ref", C.c_double),
        ("use_pml", C.c_int32), ("precision", C.c_int32), ("variant", C.c_int32),
        ("use_graph", C.c_int32), ("ckpt_every", C.c_int64),
        ("rows_per_thread", C.c_int32), ("steps_per_block", C.c_int32),
        ("block_rows", C.c_int32), ("autotune", C.c_int32),
        ("resident_segments", C.c_int32), ("resident_mem_pct", C.c_int32),
        ("tma", C.c_int32), ("reserved", C.c_int32 * 1),
    ]


class AcousticShot(C.Structure):
    _fields_ = [
        ("x0", C.c_int64), ("nx", C.c_int64), ("nstep", C.c_int64),
        ("nsrc", C.c_int64), ("srci", C.c_void_p), ("srcj", C.c_void_p),
        ("srcv", C.c_void_p), ("srcv_rows", C.c_int64),
        ("nrcv", C.c_int64), ("rcvi", C.c_void_p), ("rcvj", C.c_void_p),
    ]


class ElasticConfig(C.Structure):
    _fields_ = [
        ("NX", C.c_int64), ("NY", C.c_int64), ("NSTEP", C.c_int64),
        ("dx", C.c_double), ("dy", C.c_double), ("dt", C.c_double),
        ("npml", C.c_int64), ("npower", C.c_double), ("k_max", C.c_double),
        ("alpha_max", C.c_double), ("vp_ref", C.c_double), ("Rcoef", C.c_double),
        ("use_pml", C.c_int32), ("precision", C.c_int32), ("use_graph", C.c_int32),
        ("rows_per_warp", C.c_int32), ("ckpt_every", C.c_int64),
        ("resident_segments", C.c_int32), ("resident_mem_pct", C.c_int32),
        ("source_gradient", C.c_int32), ("autotune", C.c_int32),
        ("adjoint_passes", C.c_int32), ("reserved", C.c_int32 * 3),
    ]


class ElasticShot(C.Structure):
    _fields_ = [
        ("nsrc", C.c_int64), ("srci", C.c_void_p), ("srcj", C.c_void_p),
        ("srctype", C.c_void_p), ("srcv", C.c_void_p), ("srcv_rows", C.c_int64),
        ("nrcv", C.c_int64), ("rcvi", C.c_void_p), ("rcvj", C.c_void_p),
        ("rcvtype", C.c_void_p),
    ]


P, I64, I32, D = C.c_void_p, C.c_int64, C.c_int, C.c_double

# name -> argument types (all return int status unless listed in _RESTYPE)
_SIGS = {
    "ads_acoustic_step_fwd_f64": [P] * 7 + [D, D, D, I64, I64, P, P, P, I32, P],
    "ads_acoustic_step_fwd_f32": [P] * 7 + [D, D, D, I64, I64, P, P, P, I32, P],
    "ads_acoustic_step_bwd_f64": [P] * 15 + [D, D, D, I64, I64, P, P, P, I32, P],
    "ads_acoustic_step_bwd_f32": [P] * 15 + [D, D, D, I64, I64, P, P, P, I32, P],
    "ads_scatter_add_f64": [P, P, P, P, I64, I64, P],
    "ads_gather_f64": [P, P, P, I64, P],
    "ads_add_source_f64": [P] * 10 + [P, P, P, I64, I64, I64, P, P],
    "ads_add_source_bwd_f64": [P] * 11 + [P, P, P, I64, I64, I64, P],
    "ads_get_receive_f64": [P] * 6 + [I64, P, P, P, I64, I64, I64, P],
    "ads_get_receive_bwd_f64": [P] * 6 + [I64, P, P, P, I64, I64, I64, P],
    "ads_elastic_step_fwd_f64": [P] * 11 + [D, D, D, I64, I64, P, P, P, P, I64, P],
    "ads_elastic_step_fwd_f32": [P] * 11 + [D, D, D, I64, I64, P, P, P, P, I64, P],
    "ads_elastic_step_bwd_f64": [P] * 13 + [D, D, D, I64, I64, P],
    "ads_elastic_step_bwd_f32": [P] * 13 + [D, D, D, I64, I64, P],
    "ads_elastic_step_bwd_f64_noalloc": [P] * 13 + [D, D, D, I64, I64, P],
    "ads_acoustic_pml_profiles": [I64, I64, D, D, I64, D, D, I32, P, P],
    "ads_elastic_cpml_profiles": [I64, I64, D, D, D, I64, D, D, D, D, D, I32] + [P] * 6,
    "ads_acoustic_plan_create": [P, P, P, I64, P],
    "ads_acoustic_plan_destroy": [P],
    "ads_acoustic_plan_trace_offset": [P, I64],
    "ads_acoustic_plan_trace_count": [P],
    "ads_acoustic_plan_device_bytes": [P],
    "ads_acoustic_plan_launches": [P, I32],
    "ads_acoustic_plan_resident_segments": [P],
    "ads_acoustic_plan_steps_per_block": [P],
    "ads_acoustic_plan_profile": [P, P, P, P, P],
    "ads_acoustic_plan_forward": [P, P, P, P],
    "ads_acoustic_plan_gradient": [P, P, P, P, P, P, P],
    "ads_acoustic_plan_gradient_ex": [P, P, P, P, P, P, P, P],
    "ads_acoustic_plan_source_offset": [P, I64],
    "ads_acoustic_plan_set_source_values": [P, I64, P, P],
    "ads_acoustic_forward": [P, P, P, P, P],
    "ads_acoustic_gradient": [P, P, P, P, P, P, P],
    "ads_elastic_plan_create": [P, P, P, I64, P],
    "ads_elastic_plan_destroy": [P],
    "ads_elastic_plan_trace_offset": [P, I64],
    "ads_elastic_plan_trace_count": [P],
    "ads_elastic_plan_device_bytes": [P],
    "ads_elastic_plan_launches": [P, I32],
    "ads_elastic_plan_resident_segments": [P],
    "ads_elastic_plan_rows": [P, I32],
    "ads_acoustic_plan_tma": [P],
    "ads_acoustic_plan_rows": [P, I32],
    "ads_acoustic_plan_device_status": [P, P],
    "ads_elastic_plan_gradient_ex": [P, P, P, P, P, P, P, P, P, P, P, P],
    "ads_elastic_plan_source_offset": [P, I64],
    "ads_elastic_plan_set_source_values": [P, I64, P, P],
    "ads_elastic_plan_forward": [P, P, P, P, P, P],
    "ads_elastic_plan_gradient": [P, P, P, P, P, P, P, P, P, P, P],
    "ads_elastic_plan_profile": [P, P, P, P, P, P],
    "ads_elastic_forward": [P, P, P, P, P, P, P],
    "ads_elastic_gradient": [P, P, P, P, P, P, P, P, P, P, P],
    "ads_device_index_errors": [I32, P],
    "ads_last_error": [],
    "ads_version": [],
    "ads_launch_count": [],
}
_RESTYPE = {
    "ads_last_error": C.c_char_p,
    "ads_version": C.c_char_p,
    "ads_launch_count": C.c_int64,
    "ads_acoustic_plan_trace_offset": C.c_int64,
    "ads_acoustic_plan_source_offset": C.c_int64,
    "ads_acoustic_plan_trace_count": C.c_int64,
    "ads_acoustic_plan_device_bytes": C.c_int64,
    "ads_acoustic_plan_launches": C.c_int64,
    "ads_acoustic_plan_resident_segments": C.c_int64,
    "ads_acoustic_plan_steps_per_block": C.c_int64,
    "ads_elastic_plan_trace_offset": C.c_int64,
    "ads_elastic_plan_trace_count": C.c_int64,
    "ads_elastic_plan_device_bytes": C.c_int64,
    "ads_elastic_plan_launches": C.c_int64,
    "ads_elastic_plan_resident_segments": C.c_int64,
    "ads_elastic_plan_rows": C.c_int64,
    "ads_acoustic_plan_tma": C.c_int64,
    "ads_acoustic_plan_rows": C.c_int64,
    "ads_elastic_plan_source_offset": C.c_int64,
}
EXPORTED = sorted(_SIGS)

_lib = None


def lib():
    """Load the shared library (once); raise if it has not been built."""
    global _lib
    if _lib is None:
        if not os.path.exists(LIB_PATH):
            raise RuntimeError(
                f"{LIB_PATH} is missing: build it with __graft_entry__.build() "
                "(there is no CPU fallback)")
        L = C.CDLL(LIB_PATH)
        for name, args in _SIGS.items():
            f = getattr(L, name)
            f.argtypes = args
            f.restype = _RESTYPE.get(name, C.c_int)
        _lib = L
    return _lib


def check(rc: int) -> None:
    if rc != ADS_OK:
        raise AdsError(rc, lib().ads_last_error().decode())


def call(name: str, *args) -> None:
    check(getattr(lib(), name)(*args))
