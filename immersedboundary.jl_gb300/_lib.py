"""ctypes binding of libibgb300.so (include/ibgb300.h, include/ibgb300_ops.h).

The library is the product: every compute call goes through it.  Loading fails loudly
when the shared object is missing; there is no CPU fallback.
"""
from __future__ import annotations

import ctypes as C
import os
from pathlib import Path

import numpy as np

PKG = Path(__file__).resolve().parent
LIB_PATH = PKG / "libibgb300.so"

IB_OK = 0
IB_ERR_INVALID = 1
IB_ERR_CUDA = 2
IB_ERR_NONFINITE = 3
IB_ERR_BODY_OUT_OF_GRID = 4
IB_ERR_SINGULAR = 5
IB_ERR_CG_MAXITER = 6
IB_ERR_UNSUPPORTED = 7
IB_ERR_TIMEOUT = 8

IB_PREC_FP64 = 0
IB_PREC_MIXED = 1
IB_PREC_MIXED_TC = 2
PRECISIONS = {"fp64": IB_PREC_FP64, "mixed": IB_PREC_MIXED, "mixed_tc": IB_PREC_MIXED_TC}
IB_FORM_STOCKHAM, IB_FORM_WARP, IB_FORM_TENSOR = 0, 1, 2
IB_SCHEME_CNAB, IB_SCHEME_RKC = 0, 1
IB_MOTION_STATIC = 0
IB_MOTION_PRESCRIBED = 1
IB_WARM_PREVIOUS = 0
IB_WARM_EXTRAPOLATE = 1
IB_WARM_ZERO = 2
IB_WARM_LEARNED = 3
IB_PC_NONE = 0
IB_PC_SCHUR_REF = 1
IB_V2F_AUTO, IB_V2F_LEVELS, IB_V2F_SEQUENTIAL = 0, 1, 2

_dp = C.POINTER(C.c_double)
_ip = C.POINTER(C.c_int32)
_fp = C.POINTER(C.c_float)
_vp = C.c_void_p


class IbInfo(C.Structure):
    """Mirror of ``ib_info`` (include/ibgb300_diag.h)."""

    _fields_ = [("kernels_per_step", C.c_int32), ("nx", C.c_int32), ("ny", C.c_int32),
                ("nlevels", C.c_int32), ("nbodies", C.c_int32), ("npoints", C.c_int32),
                ("device_bytes", C.c_int64), ("setup_ms", C.c_double), ("vort2flux_order", C.c_int32),
                ("transform_form", C.c_int32), ("scheme", C.c_int32), ("rkc_stages", C.c_int32),
                ("sm_count", C.c_int32)]


class IbProblem(C.Structure):
    """Mirror of ``ib_problem`` (include/ibgb300.h)."""

    _fields_ = [
        ("nx", C.c_int32), ("ny", C.c_int32), ("nlevels", C.c_int32),
        ("x0", C.c_double), ("y0", C.c_double), ("h", C.c_double),
        ("dt", C.c_double), ("beta0", C.c_double), ("beta1", C.c_double),
        ("re", C.c_double),
        ("nbodies", C.c_int32), ("body_npoints", _ip), ("xb", _dp), ("ds", _dp),
        ("motion", C.c_int32), ("precision", C.c_int32), ("device", C.c_int32),
        ("history_capacity", C.c_int32), ("refine_sweeps", C.c_int32),
        ("scheme", C.c_int32), ("rkc_stages", C.c_int32),
    ]


# name -> (restype, argtypes); every symbol declared in include/*.h
SIGNATURES = {
    "ib_create": (C.c_int, [C.POINTER(IbProblem), C.POINTER(_vp)]),
    "ib_destroy": (C.c_int, [_vp]),
    "ib_set_state": (C.c_int, [_vp, _dp, _dp, _dp, _dp, _dp, _dp, C.c_double]),
    "ib_get_state": (C.c_int, [_vp, _dp, _dp, _dp, _dp, _dp, _dp, _dp]),
    "ib_advance": (C.c_int, [_vp, C.c_double, C.c_double, C.c_double]),
    "ib_advance_n": (C.c_int, [_vp, C.c_int32, _dp, _dp]),
    "ib_vort2flux": (C.c_int, [_vp]),
    "ib_advance_kin": (C.c_int, [_vp, C.c_double, C.c_double, C.c_double, _dp]),
    "ib_advance_n_kin": (C.c_int, [_vp, C.c_int32, _dp, _dp, _dp]),
    "ib_set_cg_options": (C.c_int, [_vp, C.c_double, C.c_int32, C.c_int32]),
    "ib_get_cg_stats": (C.c_int, [_vp, C.c_int32, _ip, _dp]),
    "ib_set_cg_preconditioner": (C.c_int, [_vp, C.c_int32, C.c_int32]),
    "ib_set_vort2flux_order": (C.c_int, [_vp, C.c_int32]),
    "ib_get_cg_preconditioner_stats": (C.c_int, [_vp, _ip, C.POINTER(C.c_int64), _dp]),
    "ib_get_body_points": (C.c_int, [_vp, _dp, _dp]),
    "ib_get_stress": (C.c_int, [_vp, _dp, _dp, _dp]),
    "ib_get_force_history": (C.c_int, [_vp, C.c_int32, _dp, _dp]),
    "ib_step_count": (C.c_int64, [_vp]),
    "ib_synchronize": (C.c_int, [_vp]),
    "ib_last_error": (C.c_char_p, [_vp]),
    "ib_status_string": (C.c_char_p, [C.c_int]),
    # operators (device pointers passed as integers)
    "ib_op_dst2": (C.c_int, [_vp, C.c_int32, _vp, _vp]),
    "ib_op_laplacian_inv": (C.c_int, [_vp, C.c_int32, _vp, _vp]),
    "ib_op_sine_lines_tc": (C.c_int, [_vp, C.c_int32, C.c_int32, _vp, _vp]),
    "ib_op_laplacian_inv_noalloc": (C.c_int, [_vp, C.c_int32, _vp, _vp]),
    "ib_op_cn_a": (C.c_int, [_vp, C.c_int32, _vp, _vp]),
    "ib_op_cn_ainv": (C.c_int, [_vp, C.c_int32, _vp, _vp]),
    "ib_op_curl": (C.c_int, [_vp, _vp, _vp, _vp]),
    "ib_op_rot": (C.c_int, [_vp, _vp, _vp]),
    "ib_op_coarsify": (C.c_int, [_vp, _vp, _vp]),
    "ib_op_get_bc": (C.c_int, [_vp, _vp, _vp]),
    "ib_op_apply_bc": (C.c_int, [_vp, _vp, _vp, C.c_double]),
    "ib_op_nonlinear": (C.c_int, [_vp, C.c_int32, _vp, C.c_double, C.c_double, _vp, _vp, _vp]),
    "ib_op_vort2flux": (C.c_int, [_vp, _vp, _vp, _vp]),
    "ib_op_reg_gather": (C.c_int, [_vp, _vp, C.c_double, C.c_double, _vp]),
    "ib_op_reg_scatter": (C.c_int, [_vp, _vp, _vp]),
    "ib_get_schur": (C.c_int, [_vp, _dp, _dp]),
    # diagnostics
    "ib_get_info": (C.c_int, [_vp, C.POINTER(IbInfo)]),
    "ib_checkpoint_save": (C.c_int, [_vp, C.c_char_p]),
    "ib_learn_set_blend": (C.c_int, [_vp, C.c_double]),
    "ib_learn_export": (C.c_int, [_vp, _fp, C.c_int64]),
    "ib_learn_import": (C.c_int, [_vp, _fp, C.c_int64]),
    "ib_checkpoint_load": (C.c_int, [_vp, C.c_char_p]),
    "ib_get_autotune": (C.c_int, [_vp, _dp, _ip]),
    "ib_advance_n_timed": (C.c_int, [_vp, C.c_int32, _dp, _dp, _dp]),
    "ib_profile_steps": (C.c_int, [_vp, C.c_int32, _dp, _dp, C.c_int32, _dp, C.POINTER(C.c_int64)]),
    "ib_measure_fp_peaks": (C.c_int, [C.c_int32, _dp, _dp]),
    "ib_profiler_start": (C.c_int, []),
    "ib_profiler_stop": (C.c_int, []),
    "ib_get_reg": (C.c_int, [_vp, _ip, _dp]),
    # learned warm start
    "ib_learn_init": (C.c_int, [_vp, C.c_int32, C.c_int32, C.c_int32, C.c_uint64]),
    "ib_learn_collect": (C.c_int, [_vp, C.c_int32]),
    "ib_learn_sample_count": (C.c_int, [_vp, _ip]),
    "ib_learn_train": (C.c_int, [_vp, C.c_int32, C.c_int32, C.c_double, C.c_uint64, _dp]),
    "ib_learn_layout": (C.c_int, [_vp, _ip, _ip, C.c_int32]),
    "ib_learn_validation": (C.c_int, [_vp, _dp, _dp]),
    "ib_learn_param_count": (C.c_int, [_vp, C.POINTER(C.c_int64)]),
    "ib_learn_get_params": (C.c_int, [_vp, _fp]),
    "ib_learn_set_params": (C.c_int, [_vp, _fp]),
    "ib_learn_gradients": (C.c_int, [_vp, C.c_int32, _fp, _fp, _fp, _dp]),
    "ib_get_cg_start_residuals": (C.c_int, [_vp, C.c_int32, _dp]),
    # ensembles
    "ib_ensemble_create": (C.c_int, [C.POINTER(_vp), C.c_int32, C.POINTER(_vp)]),
    "ib_ensemble_destroy": (C.c_int, [_vp]),
    "ib_ensemble_advance_n": (C.c_int, [_vp, C.c_int32, _dp, _dp, _dp]),
    "ib_ensemble_advance_n_kin": (C.c_int, [_vp, C.c_int32, _dp, _dp, _dp, _dp]),
    "ib_ensemble_info": (C.c_int, [_vp, _ip, _ip]),
    "ib_ensemble_set_steps_per_launch": (C.c_int, [_vp, C.c_int32]),
    "ib_ensemble_last_error": (C.c_char_p, [_vp]),
}

_LIB = None


class IBError(RuntimeError):
    """A libibgb300 call returned a non-zero status."""

    def __init__(self, status: int, message: str):
        super().__init__(f"{message} (status {status})")
        self.status = status


def load(path: str | os.PathLike | None = None):
    """Load libibgb300.so (built in-tree by ``build.py``); raises if it is absent."""
    global _LIB
    if _LIB is not None and path is None:
        return _LIB
    p = Path(path) if path else LIB_PATH
    if not p.exists():
        raise RuntimeError(
            f"{p} not found: build the CUDA library first (python -c 'import __graft_entry__ as g; g.build()')")
    lib = C.CDLL(str(p))
    for name, (res, args) in SIGNATURES.items():
        fn = getattr(lib, name)
        fn.restype = res
        fn.argtypes = args
    if path is None:
        _LIB = lib
    return lib


def dptr(a: np.ndarray | None):
    """Pointer to a C-contiguous float64 array (or NULL)."""
    if a is None:
        return None
    assert a.dtype == np.float64 and a.flags.c_contiguous
    return a.ctypes.data_as(_dp)


def fptr(a: np.ndarray | None):
    """Pointer to a C-contiguous float32 array (or NULL)."""
    if a is None:
        return None
    assert a.dtype == np.float32 and a.flags.c_contiguous
    return a.ctypes.data_as(_fp)


def iptr(a: np.ndarray | None):
    if a is None:
        return None
    assert a.dtype == np.int32 and a.flags.c_contiguous
    return a.ctypes.data_as(_ip)


def check(lib, handle, status: int):
    if status != IB_OK:
        msg = lib.ib_last_error(handle)
        raise IBError(status, (msg or b"").decode() or lib.ib_status_string(status).decode())
    return status
