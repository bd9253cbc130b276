"""ctypes binding of ``libpespace_gb300.so`` (the C ABI in include/pespace_gb300.h).

There is no CPU fallback: every call goes to the CUDA library, and loading
fails loudly when it has not been built (``python -m pespace_gb300.build``).
"""

import ctypes
import os

from . import build as _build

PES_OK = 0
PES_EINVAL = 1
PES_ENOMEM = 2
PES_ECUDA = 3
PES_ETIMEOUT = 4
PES_OPT_DENSE_STAGE = 1
PES_OPT_SAMPLE_THREADS = 2
PES_OPT_REFINE_ALL = 3
PRECISION_FP64 = 0
PRECISION_MIXED = 1
APPROX_PHENOMD = 0
APPROX_PHENOMHM = 1
MAX_DETECTORS = 4


class PesError(RuntimeError):
    """Raised when a C-ABI call returns a non-zero status."""

    def __init__(self, code, message):
        super().__init__(f"pespace_gb300 error {code}: {message}")
        self.code = code


class PesOrbit(ctypes.Structure):
    _fields_ = [
        ("kind", ctypes.c_int32),
        ("pad", ctypes.c_int32),
        ("arm_sec", ctypes.c_double),
        ("rotation_initial", ctypes.c_double),
        ("revolution_initial", ctypes.c_double),
        ("omega_revolution", ctypes.c_double),
        ("r_sec", ctypes.c_double),
        ("omega_rotation", ctypes.c_double),
        ("slam_ref", ctypes.c_double),
        ("clam_ref", ctypes.c_double),
        ("sbeta_ref", ctypes.c_double),
        ("cbeta_ref", ctypes.c_double),
        ("ck", ctypes.c_double * 3),
        ("sk", ctypes.c_double * 3),
    ]


class PesDetectorDesc(ctypes.Structure):
    _fields_ = [("orbit", PesOrbit), ("generation", ctypes.c_int32), ("pad", ctypes.c_int32)]


class PesPlanDesc(ctypes.Structure):
    _fields_ = [
        ("nbins", ctypes.c_int64),
        ("k0", ctypes.c_int64),
        ("f_step", ctypes.c_double),
        ("df", ctypes.c_double),
        ("f_ref", ctypes.c_double),
        ("cut_factor", ctypes.c_double),
        ("n_det", ctypes.c_int32),
        ("chan_mask", ctypes.c_int32),
        ("precision", ctypes.c_int32),
        ("n_sparse", ctypes.c_int32),
        ("max_batch", ctypes.c_int32),
        ("approximant", ctypes.c_int32),
        ("det", PesDetectorDesc * MAX_DETECTORS),
    ]


# name -> (restype, argtypes); mirrors include/pespace_gb300.h
_vp = ctypes.c_void_p
_d = ctypes.c_double
_i32 = ctypes.c_int32
_i64 = ctypes.c_int64
SIGNATURES = {
    "pes_last_error": (ctypes.c_char_p, []),
    "pes_version": (ctypes.c_int, []),
    "pes_orbit_vectors": (ctypes.c_int, [ctypes.POINTER(PesOrbit), _vp, _i64, _vp, _vp]),
    "pes_polarization": (ctypes.c_int, [_d, _d, _d, _vp, _vp, _vp]),
    "pes_response_links": (ctypes.c_int, [ctypes.POINTER(PesOrbit), _vp, _i64, _i32, _vp, _vp, _vp, _d, _d, _d, _d,
                                          _vp, _vp]),
    "pes_tdi_combination": (ctypes.c_int, [_vp, _i64, _d, _i32, _i32, _vp, _vp, _vp]),
    "pes_whittle_workspace_len": (_i64, [_i64]),
    "pes_whittle_lnl": (ctypes.c_int, [_vp, _vp, _vp, _i32, _i64, _d, _vp, _i64, _vp, _vp]),
    "pes_whittle_lnl_noalloc": (ctypes.c_int, [_vp, _vp, _vp, _i32, _i64, _d, _vp, _vp]),
    "pes_phenomd": (ctypes.c_int, [_vp, _vp, _i64, _d, _d, _vp, _vp, _vp, _vp]),
    "pes_phenomhm": (ctypes.c_int, [_vp, _vp, _i64, _d, _d, _vp, _vp, _vp, _vp]),
    "pes_pn_tf": (ctypes.c_int, [_vp, _i64, _vp, _i64, _vp, _vp]),
    "pes_td_tdi_combination": (ctypes.c_int, [_vp, _i64, _i64, _i64, _d, _d, _i32, _i32, _vp, _vp]),
    "pes_td_tdi_layout": (ctypes.c_int, [_d, _d, _i32, _vp, _vp, _vp, _vp]),
    "pes_td_tdi_combination_mixed": (ctypes.c_int, [_vp, _i64, _i64, _i64, _d, _d, _i32, _i32, _vp, _vp]),
    "pes_plan_create": (ctypes.c_int, [ctypes.POINTER(PesPlanDesc), ctypes.POINTER(_vp)]),
    "pes_plan_destroy": (ctypes.c_int, [_vp]),
    "pes_plan_set_data": (ctypes.c_int, [_vp, _i32, _vp, _vp, _vp]),
    "pes_lnl_batch": (ctypes.c_int, [_vp, _vp, _i64, _vp, _vp, _vp]),
    "pes_lnl_grad_batch": (ctypes.c_int, [_vp, _vp, _i64, _vp, _vp, _vp, _vp]),
    "pes_plan_model_tdi": (ctypes.c_int, [_vp, _i32, _i32, _vp, _vp, _vp]),
    "pes_plan_profile": (ctypes.c_int, [_vp, _i32]),
    "pes_plan_stats": (ctypes.c_int, [_vp, _vp, _vp]),
    "pes_plan_set_option": (ctypes.c_int, [_vp, _i32, _i64]),
    "pes_plan_get_option": (ctypes.c_int, [_vp, _i32, _vp]),
    "pes_kernel_class_name": (ctypes.c_char_p, [_i32]),
    "pes_plan_work": (ctypes.c_int, [_vp, _i64, _vp, _vp]),
    "pes_fisher_batch": (ctypes.c_int, [_vp, _vp, _i64, _vp, _vp, _vp]),
}
KERNEL_CLASSES = 8

_lib = None


def library_path():
    return _build.LIB


def load():
    """Load the CUDA library (building it first if the sources are newer)."""
    global _lib
    if _lib is None:
        path = _build.LIB
        if not os.path.exists(path):
            raise RuntimeError(
                f"pespace_gb300 CUDA library not built ({path}); run `python -m pespace_gb300.build`"
            )
        lib = ctypes.CDLL(path)
        for name, (res, args) in SIGNATURES.items():
            fn = getattr(lib, name)
            fn.restype = res
            fn.argtypes = args
        _lib = lib
    return _lib


def check(code):
    if code != PES_OK:
        msg = load().pes_last_error()
        raise PesError(code, msg.decode() if msg else "")
    return code


def ptr(t):
    """Device (or host) address of a tensor / array as a ctypes void pointer."""
    if t is None:
        return None
    if hasattr(t, "data_ptr"):
        return ctypes.c_void_p(t.data_ptr())
    return t.ctypes.data_as(ctypes.c_void_p)


def stream_handle(stream=None):
    import torch

    s = stream if stream is not None else torch.cuda.current_stream()
    return ctypes.c_void_p(s.cuda_stream)
