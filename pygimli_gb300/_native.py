"""ctypes binding of libertgb.so (the C ABI in include/ertgb.h).

The library is built in-tree by pygimli_gb300/build.py.  There is no CPU or
PyTorch fallback: if the library is missing or no CUDA device is present,
loading fails with an error.
"""
from __future__ import annotations

import ctypes
import os

from . import build as _build

OK, BAD_INPUT, NOT_CONVERGED, OOM, CUDA_ERROR, STATE = range(6)
_STATUS = {BAD_INPUT: ValueError, NOT_CONVERGED: RuntimeError, OOM: MemoryError,
           CUDA_ERROR: RuntimeError, STATE: RuntimeError}


class ErtgbError(RuntimeError):
    def __init__(self, code, msg):
        super().__init__(f"ertgb status {code}: {msg}")
        self.code = code


class Stats(ctypes.Structure):
    _fields_ = [("iterations", ctypes.c_int32), ("n_rhs", ctypes.c_int32),
                ("max_rel_residual", ctypes.c_double), ("ms_assemble", ctypes.c_double),
                ("ms_rhs", ctypes.c_double), ("ms_solve", ctypes.c_double),
                ("ms_collect", ctypes.c_double), ("ms_jacobian", ctypes.c_double),
                ("launches_response", ctypes.c_int64), ("launches_jacobian", ctypes.c_int64),
                ("stalled_columns", ctypes.c_int32)]


class BatchInfo(ctypes.Structure):
    _fields_ = [("rows_per_tile", ctypes.c_int32), ("rhs_width", ctypes.c_int32),
                ("n_candidates", ctypes.c_int32), ("cached", ctypes.c_int32),
                ("cand_rows", ctypes.c_int32 * 16), ("cand_width", ctypes.c_int32 * 16),
                ("cand_ms", ctypes.c_double * 16), ("spmm_tiles", ctypes.c_int64),
                ("vector_tiles", ctypes.c_int64), ("columns", ctypes.c_int64),
                ("iterations", ctypes.c_int32), ("stalled_columns", ctypes.c_int32),
                ("launches", ctypes.c_int64), ("ms_assemble", ctypes.c_double),
                ("ms_solve", ctypes.c_double), ("ms_collect", ctypes.c_double)]


# name -> (restype, argtypes)
_vp, _i32, _i64, _d = ctypes.c_void_p, ctypes.c_int32, ctypes.c_int64, ctypes.c_double
_ci = ctypes.c_int
SIGNATURES = {
    "ertgb_create": (_ci, [ctypes.POINTER(_vp), _ci]),
    "ertgb_destroy": (_ci, [_vp]),
    "ertgb_last_error": (ctypes.c_char_p, [_vp]),
    "ertgb_set_mesh": (_ci, [_vp, _ci, _ci, _ci, _vp, _ci, _vp, _vp, _ci, _vp, _vp, _vp]),
    "ertgb_set_electrodes": (_ci, [_vp, _ci, _vp, _d]),
    "ertgb_set_kw": (_ci, [_vp, _ci, _vp, _vp]),
    "ertgb_set_primary": (_ci, [_vp, _ci, _ci, _i64, _vp]),
    "ertgb_set_electrode_shapes": (_ci, [_vp, _ci, _vp, _vp]),
    "ertgb_set_reference": (_ci, [_vp, _ci, _ci, _ci, _vp]),
    "ertgb_analytic_potentials": (_ci, [_vp, _d]),
    "ertgb_set_scheme": (_ci, [_vp, _ci, _vp, _vp]),
    "ertgb_set_solver": (_ci, [_vp, _d, _ci, _ci]),
    "ertgb_set_precision": (_ci, [_vp, _ci]),
    "ertgb_set_formulation": (_ci, [_vp, _ci]),
    "ertgb_set_extension": (_ci, [_vp, _ci, ctypes.c_int64, _vp, _vp, _vp, _vp, _vp, _ci]),
    "ertgb_response": (_ci, [_vp, _vp, _vp, _vp]),
    "ertgb_response_host": (_ci, [_vp, _vp, _vp]),
    "ertgb_jacobian": (_ci, [_vp, _vp, _ci, _vp, _ci, _vp]),
    "ertgb_jacobian_host": (_ci, [_vp, _vp, _ci, _vp, _ci]),
    "ertgb_sizes": (_ci, [_vp, ctypes.POINTER(_i64), ctypes.POINTER(_i64), ctypes.POINTER(_i64),
                          ctypes.POINTER(_i64)]),
    "ertgb_get_pattern": (_ci, [_vp, _vp, _vp]),
    "ertgb_get_matrix": (_ci, [_vp, _ci, _ci, _vp]),
    "ertgb_get_potentials": (_ci, [_vp, _vp]),
    "ertgb_get_electrode_potentials": (_ci, [_vp, _vp]),
    "ertgb_get_primary": (_ci, [_vp, _vp]),
    "ertgb_get_stats": (_ci, [_vp, ctypes.POINTER(Stats)]),
    "ertgb_csr_spmm_dot": (_ci, [_i64, _i64, _vp, _vp, _vp, _ci, _ci, _i64, _vp, _vp, _vp, _vp]),
    "ertgb_csr_spmm_dot_noalloc": (_ci, [_i64, _i64, _vp, _vp, _vp, _ci, _ci, _i64, _vp, _vp, _vp, _vp]),
    "ertgb_profile_kernel": (_ci, [_vp, _ci, _ci, _vp, ctypes.POINTER(_d), ctypes.POINTER(_d),
                                   ctypes.POINTER(_d)]),
    "ertgb_set_precond_weights": (_ci, [_vp, _vp, _i64]),
    "ertgb_assemble": (_ci, [_vp, _vp, _vp]),
    "ertgb_lp_forward": (_ci, [_vp, _vp, _vp, _vp]),
    "ertgb_lp_loss_grad": (_ci, [_vp, _vp, _vp, ctypes.POINTER(_d), _vp]),
    "ertgb_lp_adam": (_ci, [_vp, _vp, _vp, _vp, _i64, _d, _d, _d, _d, _ci, _d, _vp]),
    "ertgb_lp_features": (_ci, [_vp, _vp, _vp, _vp]),
    "ertgb_batch_response": (_ci, [_vp, _ci, _vp, _vp, ctypes.POINTER(BatchInfo), _vp]),
    "ertgb_cgls": (_ci, [_vp, _ci, _i64, _i64, _i64, _vp, _vp, _vp, _vp, _vp, _vp, _vp, _vp, _vp, _vp, _vp, _vp,
                         _vp, _d, _vp, _ci, _d, ctypes.POINTER(_i32), _vp]),
    "ertgb_response_complex": (_ci, [_vp, _vp, _vp, _vp, _vp, _vp]),
    "ertgb_jacobian_complex": (_ci, [_vp, _vp, _vp, _ci, _vp, _vp]),
    "ertgb_refine": (_ci, [_ci, _ci, _ci, _i64, _vp, _vp, _i64, _vp, _vp, _i64, _vp, _vp, _vp, ctypes.POINTER(_vp)]),
    "ertgb_refined_sizes": (_ci, [_vp] + [ctypes.POINTER(_i64)] * 5),
    "ertgb_refined_get": (_ci, [_vp] * 8),
    "ertgb_refined_free": (_ci, [_vp]),
}

LP_NPARAM = 83202

_lib = None


def lib_path():
    return _build.LIB


def load(build_if_missing=False):
    """Load libertgb.so and declare every exported signature."""
    global _lib
    if _lib is not None:
        return _lib
    path = lib_path()
    if not os.path.exists(path):
        if build_if_missing:
            _build.build()
        else:
            raise ImportError(f"libertgb.so not built ({path}); run pygimli_gb300.build.build()")
    L = ctypes.CDLL(path)
    for name, (res, args) in SIGNATURES.items():
        f = getattr(L, name)
        f.restype = res
        f.argtypes = args
    _lib = L
    return L


def check(ctx, rc):
    if rc != OK:
        msg = load().ertgb_last_error(ctx)
        raise ErtgbError(rc, msg.decode() if msg else "")
    return rc
