"""ctypes binding of libqmlg.so (the C ABI declared in include/qmlg.h).

The library is the only compute path: if it is missing or cannot be loaded the
import fails loudly; there is no CPU fallback.
"""
from __future__ import annotations

import ctypes
import os

from . import build as _build

_HERE = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = _build.LIB

QMLG_OK = 0
QMLG_E_ARG = -1
QMLG_E_CUDA = -2
QMLG_E_WORKSPACE = -3
QMLG_E_TOO_MANY_ATOMS = -4
QMLG_E_NOT_CONVERGED = -5
QMLG_E_TIMEOUT = -6
QMLG_E_TOO_LARGE = -7

QMLG_KERNEL_SYMMETRIC = 1
QMLG_KIND_GAUSSIAN = 0
QMLG_KIND_LAPLACIAN = 1
QMLG_PREC_FP64 = 0
QMLG_PREC_MIXED = 1

_ERRORS = {
    QMLG_E_ARG: "invalid argument",
    QMLG_E_CUDA: "CUDA error",
    QMLG_E_WORKSPACE: "workspace missing or too small",
    QMLG_E_TOO_MANY_ATOMS: "a molecule has more atoms than size (or than 32)",
    QMLG_E_NOT_CONVERGED: "refinement did not converge",
    QMLG_E_TIMEOUT: "a bounded device wait gave up",
    QMLG_E_TOO_LARGE: "problem exceeds a fixed-size internal buffer",
}


class QmlgError(RuntimeError):
    def __init__(self, status, where):
        msg = "%s failed: %s (status %d)" % (where, _ERRORS.get(status, "error"), status)
        if status == QMLG_E_CUDA and _lib is not None:
            msg += ": " + _lib.qmlg_last_error().decode()
        super().__init__(msg)
        self.status = status


class QmlgSolveReport(ctypes.Structure):
    _fields_ = [("precision_used", ctypes.c_int), ("info", ctypes.c_int),
                ("outer_iterations", ctypes.c_int), ("inner_iterations", ctypes.c_int),
                ("fell_back", ctypes.c_int), ("shift", ctypes.c_double),
                ("backward_error", ctypes.c_double), ("last_correction", ctypes.c_double)]

    def as_dict(self):
        return {name: getattr(self, name) for name, _ in self._fields_}


class QmlgRefineOpts(ctypes.Structure):
    _fields_ = [("max_outer", ctypes.c_int), ("max_inner", ctypes.c_int), ("tol", ctypes.c_double),
                ("shift", ctypes.c_double), ("allow_fallback", ctypes.c_int),
                ("slices", ctypes.c_int)]


class QmlgBatchProblem(ctypes.Structure):
    _fields_ = [("X", ctypes.c_void_p), ("ldx", ctypes.c_int64), ("n", ctypes.c_int),
                ("kind", ctypes.c_int), ("sigma", ctypes.c_double), ("lam", ctypes.c_double),
                ("y", ctypes.c_void_p), ("alpha", ctypes.c_void_p), ("K", ctypes.c_void_p),
                ("status", ctypes.c_void_p), ("correction", ctypes.c_void_p)]


_P = ctypes.c_void_p
_I = ctypes.c_int
_I64 = ctypes.c_int64
_D = ctypes.c_double
_SZ = ctypes.c_size_t

# name -> (restype, argtypes); every symbol include/qmlg.h declares
SIGNATURES = {
    "qmlg_version": (ctypes.c_char_p, []),
    "qmlg_last_error": (ctypes.c_char_p, []),
    "qmlg_launch_count": (ctypes.c_uint64, []),
    "qmlg_set_thread_sm_limit": (None, [_I]),
    "qmlg_set_thread_persistent": (None, [_I]),
    "qmlg_set_thread_cooperative": (None, [_I]),
    "qmlg_coulomb_matrix": (_I, [_P, _P, _P, _I, _I, _I, _P, _P, _P]),
    "qmlg_gaussian_kernel": (_I, [_P, _I64, _I, _P, _I64, _I, _I, _D, _P, _I64, _I, _D, _P]),
    "qmlg_laplacian_kernel": (_I, [_P, _I64, _I, _P, _I64, _I, _I, _D, _P, _I64, _I, _D, _P]),
    "qmlg_atomic_coulomb_matrix": (_I, [_P, _P, _P, _I, _P, _P, _I, _I, _I, _D, _D, _D, _D, _P, _P,
                                        _P]),
    "qmlg_local_kernels": (_I, [_I, _P, _I64, _P, _I, _P, _I64, _P, _I, _I, _P, _I, _P, _I, _P]),
    "qmlg_local_kernels_emulated_workspace_size": (_SZ, [_I, _I64, _I64, _I, _I]),
    "qmlg_local_kernels_emulated": (_I, [_I, _P, _I64, _P, _I, _P, _I64, _P, _I, _I, _P, _I, _P,
                                         _I, _P, _SZ, _P]),
    "qmlg_cho_invert_workspace_size": (_SZ, [_I, _I]),
    "qmlg_cho_invert": (_I, [_P, _I, _I64, _P, _I64, _I, _P, _SZ, _P]),
    "qmlg_bkf_solve_workspace_size": (_SZ, [_I]),
    "qmlg_bkf_solve": (_I, [_P, _I, _I64, _P, _P, _P, _SZ, _P]),
    "qmlg_bkf_invert_workspace_size": (_SZ, [_I]),
    "qmlg_bkf_invert": (_I, [_P, _I, _I64, _P, _I64, _P, _SZ, _P]),
    "qmlg_linear_kernel": (_I, [_P, _I64, _I, _P, _I64, _I, _I, _P, _I64, _I, _D, _P]),
    "qmlg_matern_kernel_l2": (_I, [_P, _I64, _I, _P, _I64, _I, _I, _D, _I, _P, _I64, _I, _D, _P]),
    "qmlg_sargan_kernel": (_I, [_P, _I64, _I, _P, _I64, _I, _I, _D, _P, _I, _P, _I64, _I, _D,
                                _P]),
    "qmlg_gaussian_kernel_emulated_workspace_size": (_SZ, [_I, _I, _I, _I]),
    "qmlg_gaussian_kernel_emulated": (_I, [_P, _I64, _I, _P, _I64, _I, _I, _D, _P, _I64, _I, _D,
                                           _P, _SZ, _P]),
    "qmlg_predict_emulated_workspace_size": (_SZ, [_I, _I, _I]),
    "qmlg_predict_emulated": (_I, [_P, _I64, _I, _P, _I64, _I, _I, _D, _P, _P, _P, _SZ, _P]),
    "qmlg_predict_emulated_async": (_I, [_P, _I64, _I, _P, _I64, _I, _I, _D, _P, _P, _P, _P,
                                         _SZ, _P]),
    "qmlg_sargan_kernel_fixed_workspace_size": (_SZ, [_I, _I, _I, _I]),
    "qmlg_sargan_kernel_fixed": (_I, [_P, _I64, _I, _P, _I64, _I, _I, _D, _P, _I, _P, _I64, _I, _D,
                                      _P, _SZ, _P]),
    "qmlg_matern_kernel_l2_emulated_workspace_size": (_SZ, [_I, _I, _I, _I]),
    "qmlg_matern_kernel_l2_emulated": (_I, [_P, _I64, _I, _P, _I64, _I, _I, _D, _I, _P, _I64, _I,
                                            _D, _P, _SZ, _P]),
    "qmlg_linear_kernel_emulated_workspace_size": (_SZ, [_I, _I, _I, _I]),
    "qmlg_linear_kernel_emulated": (_I, [_P, _I64, _I, _P, _I64, _I, _I, _P, _I64, _I, _D, _P,
                                         _SZ, _P]),
    "qmlg_laplacian_kernel_fixed_workspace_size": (_SZ, [_I, _I, _I, _I]),
    "qmlg_laplacian_kernel_fixed": (_I, [_P, _I64, _I, _P, _I64, _I, _I, _D, _P, _I64, _I, _D,
                                         _P, _SZ, _P]),
    "qmlg_predict_gemv": (_I, [_P, _I64, _I, _I, _P, _P, _P]),
    "qmlg_predict_workspace_size": (_SZ, [_I, _I]),
    "qmlg_predict_fused": (_I, [_I, _P, _I64, _I, _P, _I64, _I, _I, _D, _P, _P, _P, _SZ, _P]),
    "qmlg_predict_fused_noalloc": (_I, [_I, _P, _I64, _I, _P, _I64, _I, _I, _D, _P, _P, _P]),
    "qmlg_epilogue_exp": (_I, [_P, _P, _I, _P]),
    "qmlg_cholesky_workspace_size": (_SZ, [_I]),
    "qmlg_cholesky": (_I, [_P, _I, _I64, _D, _P, _SZ, _P]),
    "qmlg_cholesky_mixed_workspace_size": (_SZ, [_I]),
    "qmlg_cholesky_mixed": (_I, [_P, _I, _I64, _D, _P, _SZ, _P]),
    "qmlg_syrk_emulated_workspace_size": (_SZ, [_I, _I]),
    "qmlg_syrk_emulated": (_I, [_P, _I64, _I, _P, _I64, _I, _P, _SZ, _P]),
    "qmlg_cholesky_solve_factored": (_I, [_P, _I, _I64, _P, _P, _P]),
    "qmlg_solve_workspace_size": (_SZ, [_I, _I]),
    "qmlg_solve": (_I, [_P, _I, _I64, _P, _P, _D, _I, ctypes.POINTER(QmlgRefineOpts),
                        ctypes.POINTER(QmlgSolveReport), _P, _SZ, _P]),
    "qmlg_gaussian_kernel_emulated_async": (_I, [_P, _I64, _I, _P, _I64, _I, _I, _D, _P, _I64,
                                                 _I, _D, _P, _P, _SZ, _P]),
    "qmlg_solve_async_workspace_size": (_SZ, [_I]),
    "qmlg_solve_async": (_I, [_P, _I, _I64, _P, _P, _D, _I, _P, _P, _P, _SZ, _P]),
    "qmlg_residual_workspace_size": (_SZ, [_I]),
    "qmlg_residual_dd": (_I, [_P, _I, _I64, _P, _D, _P, _P, _P, _P, _SZ, _P]),
    "qmlg_predict_laplacian_fixed_workspace_size": (_SZ, [_I, _I, _I]),
    "qmlg_predict_laplacian_fixed": (_I, [_P, _I64, _I, _P, _I64, _I, _I, _D, _P, _P, _P, _SZ, _P]),
    "qmlg_predict_laplacian_fixed_async": (_I, [_P, _I64, _I, _P, _I64, _I, _I, _D, _P, _P, _P, _P,
                                                _SZ, _P]),
    "qmlg_laplacian_kernel_fixed_async": (_I, [_P, _I64, _I, _P, _I64, _I, _I, _D, _P, _I64, _I,
                                               _D, _P, _P, _SZ, _P]),
    "qmlg_fit_batched_workspace_size": (_SZ, [ctypes.POINTER(QmlgBatchProblem), _I, _I]),
    "qmlg_fit_batched_async": (_I, [ctypes.POINTER(QmlgBatchProblem), _I, _I, _I, _I, _I, _P, _SZ,
                                    _P]),
    "qmlg_selftest_wait_timeout_workspace_size": (_SZ, []),
    "qmlg_selftest_wait_timeout": (_I, [_P, _SZ, _P]),
    "qmlg_read_files": (_I, [_P, _I, _I, _P, _P, _P, _P]),
    "qmlg_parse_xyz": (_I, [_P, _P, _I, _I, _P, _P, _P, _P, _I64]),
}

_lib = None


def load(build_if_missing: bool = True):
    """Load libqmlg.so (building it first if it is absent and nvcc is present)."""
    global _lib
    if _lib is not None:
        return _lib
    if not os.path.exists(LIB_PATH) and build_if_missing:
        _build.build()
    if not os.path.exists(LIB_PATH):
        raise ImportError("libqmlg.so not found at %s; run qml_gb300.build.build()" % LIB_PATH)
    lib = ctypes.CDLL(LIB_PATH)
    for name, (res, args) in SIGNATURES.items():
        fn = getattr(lib, name)
        fn.restype = res
        fn.argtypes = args
    _lib = lib
    return lib


def check(status, where):
    if status < 0:
        raise QmlgError(status, where)
    return status
