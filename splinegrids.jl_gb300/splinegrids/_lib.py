"""ctypes binding of libsplinegrids_b200.so (declared in include/splinegrids_b200.h).

The library is the only compute path of this package: there is no CPU fallback.
Loading fails loudly when the library has not been built or CUDA is unavailable.
"""
from __future__ import annotations

import ctypes as C
import os

import torch

_HERE = os.path.dirname(os.path.abspath(__file__))
_PKG_ROOT = os.path.dirname(_HERE)
LIB_PATH = os.path.join(_PKG_ROOT, "lib", "libsplinegrids_b200.so")

SG_OK = 0
SG_ERR_INVALID_ARGUMENT = 1
SG_ERR_UNSUPPORTED = 2
SG_ERR_CUDA = 3
SG_ERR_TIMEOUT = 4
SG_ERR_OUT_OF_MEMORY = 5
SG_ERR_DEVICE_CHECK = 6

SG_F64 = 0
SG_F32 = 1
SG_BF16_F32 = 2

SG_MAX_NIN = 8
SG_MAX_DEGREE = 15

_STATUS_NAMES = {
    1: "invalid argument", 2: "unsupported", 3: "CUDA error", 4: "timeout",
    5: "out of memory", 6: "device check failed",
}


class SplineGridsError(RuntimeError):
    """Raised when a library call returns a status other than SG_OK."""

    def __init__(self, code: int, message: str):
        super().__init__(f"{message} [{_STATUS_NAMES.get(code, code)}]")
        self.code = code
        self.message = message


class GridDesc(C.Structure):
    _fields_ = [
        ("nin", C.c_int32), ("nout", C.c_int32), ("dtype", C.c_int32), ("has_weights", C.c_int32),
        ("n_samples", C.c_int64 * SG_MAX_NIN), ("n_basis", C.c_int64 * SG_MAX_NIN),
        ("degree", C.c_int32 * SG_MAX_NIN), ("max_derivative_order", C.c_int32 * SG_MAX_NIN),
        ("sample_indices", C.c_void_p * SG_MAX_NIN), ("basis_eval", C.c_void_p * SG_MAX_NIN),
    ]


class RefMat(C.Structure):
    _fields_ = [
        ("m", C.c_int64), ("n", C.c_int64), ("nnz", C.c_int64),
        ("row_pointer", C.c_void_p), ("column_start", C.c_void_p), ("nzval", C.c_void_p),
    ]


_vp = C.c_void_p
_i32 = C.c_int32
_i64 = C.c_int64
_pi64 = C.POINTER(C.c_int64)
_pi32 = C.POINTER(C.c_int32)

# name -> (restype, argtypes); the full exported surface of the header
SIGNATURES = {
    "sg_version": (C.c_int, []),
    "sg_last_error": (C.c_char_p, []),
    "sg_expand_knots": (C.c_int, [_i32, _vp, _vp, _i64, _i64, _vp, _vp]),
    "sg_sample_indices": (C.c_int, [_i32, _vp, _i64, _vp, _i64, _i32, _vp, _vp]),
    "sg_basis_eval": (C.c_int, [_i32, _vp, _i64, _vp, _vp, _i64, _i32, _i32, _vp, _vp]),
    "sg_decompress": (C.c_int, [_i32, _vp, _vp, _i64, _i32, _i32, _i32, _i64, _vp, _vp]),
    "sg_grid_plan_create": (C.c_int, [C.POINTER(GridDesc), _vp, C.POINTER(_vp)]),
    "sg_grid_plan_refresh": (C.c_int, [_vp, _vp]),
    "sg_grid_plan_destroy": (None, [_vp]),
    "sg_grid_plan_workspace_bytes": (C.c_int64, [_vp]),
    "sg_grid_plan_enable_timing": (C.c_int, [_vp, _i32]),
    "sg_grid_plan_pass_times": (C.c_int, [_vp, C.POINTER(C.c_float), _pi32]),
    "sg_grid_plan_check": (C.c_int, [_vp, _vp]),
    "sg_evaluate": (C.c_int, [_vp, _pi32, _vp, _vp, _vp, _vp]),
    "sg_evaluate_adjoint": (C.c_int, [_vp, _pi32, _vp, _vp, _vp]),
    "sg_mult": (C.c_int, [_i32, _i32, _pi64, _pi64, _i32, C.POINTER(RefMat), _pi32, _vp, _vp, _vp]),
    "sg_mult_adjoint": (C.c_int, [_i32, _i32, _pi64, _pi64, _i32, C.POINTER(RefMat), _pi32, _vp, _vp,
                                  _vp]),
    "sg_local_refinement": (C.c_int, [_i32, _i32, _i32, _pi64, _i64, _vp, _vp, _vp, _vp]),
    "sg_local_refinement_adjoint": (C.c_int, [_i32, _i32, _i32, _pi64, _i64, _vp, _vp, _vp, _vp]),
    "sg_evaluate_noalloc": (C.c_int, [C.POINTER(GridDesc), _pi32, _vp, _vp, _vp, _vp]),
    "sg_batch_plan_create": (C.c_int, [_i32, C.POINTER(GridDesc), _pi32, _vp, C.POINTER(_vp)]),
    "sg_batch_set_arrays": (C.c_int, [_vp, C.POINTER(_vp), C.POINTER(_vp), C.POINTER(_vp),
                                      C.POINTER(_vp)]),
    "sg_batch_run": (C.c_int, [_vp, _i32, _vp]),
    "sg_batch_enable_profile": (C.c_int, [_vp, _i32]),
    "sg_batch_profile": (C.c_int, [_vp, _vp, _pi64]),
    "sg_evaluate_multi": (C.c_int, [_vp, _i32, _pi32, _vp, _vp, C.POINTER(_vp), _vp]),
    "sg_select_workspace_bytes": (C.c_int64, [_i64]),
    "sg_sum_outputs": (C.c_int, [_i32, _i64, _i32, _vp, _vp, _vp, _vp, _vp]),
    "sg_select_above": (C.c_int, [_i32, _i32, _pi64, _i32, _vp, _vp, C.c_double, _vp, _i64, _vp,
                                  _vp, _vp, _pi64, _vp, _vp]),
    "sg_select_rows": (C.c_int, [_i32, _i64, _vp, _i32, _vp, _i32, _vp, _vp, _vp, _pi64, _vp, _vp]),
    "sg_refine_matrix_workspace_bytes": (C.c_int64, [_i32, _i32, _i64, _i64]),
    "sg_refine_matrix": (C.c_int, [_i32, _i32, _vp, _i64, _i64, _vp, _vp, _vp, _vp, _vp, _pi64,
                                   _vp, _vp]),
    "sg_copy_list": (C.c_int, [_i64, C.POINTER(_vp), C.POINTER(_vp), _pi64, _vp]),
    "sg_grid_plan_tune": (C.c_int, [_vp, _pi32, _vp, _vp, _vp, _pi32]),
    "sg_grid_plan_untune": (C.c_int, [_vp]),
    "sg_grid_plan_set_strategy": (C.c_int, [_vp, _i32]),
    "sg_grid_plan_paths": (C.c_int, [_vp, _pi32, _pi32]),
    "sg_batch_set_strategy": (C.c_int, [_vp, _i32]),
    "sg_batch_fused_grids": (C.c_int64, [_vp]),
    "sg_batch_tune": (C.c_int, [_vp, _vp, _pi64]),
    "sg_batch_set_unit_sizes": (C.c_int, [_vp, _i64, _i64]),
    "sg_lsqr_create": (C.c_int, [_i32, _i64, _i64, _vp, _vp, _vp, _vp, _vp, _vp, C.c_double,
                                 C.c_double, C.c_double, C.c_double, _i64, C.POINTER(_vp)]),
    "sg_lsqr_destroy": (C.c_int, [_vp]),
    "sg_lsqr_start": (C.c_int, [_vp, _vp, _vp]),
    "sg_lsqr_after_forward": (C.c_int, [_vp, _vp]),
    "sg_lsqr_after_adjoint": (C.c_int, [_vp, _vp]),
    "sg_lsqr_capture_begin": (C.c_int, [_vp, _vp]),
    "sg_lsqr_capture_body": (C.c_int, [_vp, _vp, C.POINTER(_vp)]),
    "sg_lsqr_capture_end": (C.c_int, [_vp, _vp]),
    "sg_lsqr_launch": (C.c_int, [_vp, _vp]),
    "sg_lsqr_info": (C.c_int, [_vp, _vp, _pi64, C.POINTER(C.c_double)]),
    "sg_batch_check": (C.c_int, [_vp, _vp]),
    "sg_batch_plan_destroy": (None, [_vp]),
    "sg_batch_plan_workspace_bytes": (C.c_int64, [_vp]),
    "sg_batch_items": (C.c_int64, [_vp, _i32]),
    "sg_fit_plan_create": (C.c_int, [_i32, _i32, _vp, _vp, _vp, _pi64, C.POINTER(C.c_double), _i32,
                                     _vp, _pi64, _pi32, _vp, C.POINTER(_vp)]),
    "sg_fit_plan_destroy": (C.c_int, [_vp]),
    "sg_fit_loss": (C.c_int, [_vp, _vp]),
    "sg_fit_update": (C.c_int, [_vp, C.c_double, _vp]),
    "sg_fit_losses": (C.c_int, [_vp, _vp, C.POINTER(C.c_double), _pi64, C.POINTER(C.c_double), _i64]),
    "sg_test_fail_allocations": (C.c_int, [_i64]),
    "sg_test_live_allocations": (C.c_int64, []),
    "sg_test_set_wait_limits": (C.c_int, [_i64, _i64]),
    "sg_test_block_waits": (C.c_int, [_i32, _i32]),
}

_lib = None


def load(path: str = LIB_PATH):
    """Load the library (once) and declare every exported signature."""
    global _lib
    if _lib is not None:
        return _lib
    if not os.path.exists(path):
        raise RuntimeError(
            f"{path} is missing: build it with `python splinegrids.jl_gb300/build.py` "
            "(needs nvcc); this package has no CPU fallback")
    lib = C.CDLL(path)
    for name, (res, args) in SIGNATURES.items():
        fn = getattr(lib, name)
        fn.restype = res
        fn.argtypes = args
    _lib = lib
    return lib


def last_error() -> str:
    return (load().sg_last_error() or b"").decode(errors="replace")


def check(rc: int) -> None:
    if rc != SG_OK:
        raise SplineGridsError(rc, last_error())


def stream_handle(device: torch.device | None = None) -> int:
    """The current torch CUDA stream of `device` as a cudaStream_t value."""
    return torch.cuda.current_stream(device).cuda_stream


def i64_array(vals):
    return (C.c_int64 * max(1, len(vals)))(*[int(v) for v in vals])


def i32_array(vals):
    return (C.c_int32 * max(1, len(vals)))(*[int(v) for v in vals])
