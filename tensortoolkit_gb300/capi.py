"""ctypes declarations of include/qltg.h (the C ABI of libqltg.so)."""
from __future__ import annotations

import ctypes as C
import os
import re

from . import _native

QLTG_OK, QLTG_ERR_INVALID, QLTG_ERR_CUDA, QLTG_ERR_OOM, QLTG_ERR_TIMEOUT, QLTG_ERR_NOCONV, \
    QLTG_ERR_EMPTY_SVD, QLTG_ERR_UNSUPPORTED, QLTG_ERR_LAYOUT = range(9)
QLTG_SIDE_HEAD, QLTG_SIDE_TAIL = 0, 1
QLTG_F64, QLTG_C128 = 0, 1
QLTG_MODE_FP64, QLTG_MODE_SPLIT = 0, 1

HEADER = os.path.join(_native.ROOT, "include", "qltg.h")


class TensorDesc(C.Structure):
    _fields_ = [("rank", C.c_int32), ("dtype", C.c_int32), ("qn_ncomp", C.c_int32), ("parity_comp", C.c_int32),
                ("dirs", C.c_void_p), ("nsct", C.c_void_p), ("qns", C.c_void_p), ("dims", C.c_void_p),
                ("nblk", C.c_int64), ("coords", C.c_void_p)]


_P = C.c_void_p
_I64P = C.POINTER(C.c_int64)
_SIGS = {
    "qltg_create": ([C.c_int, C.POINTER(_P)], C.c_int),
    "qltg_destroy": ([_P], C.c_int),
    "qltg_last_error": ([], C.c_char_p),
    "qltg_ctrct_plan_create": ([_P, C.POINTER(TensorDesc), C.POINTER(TensorDesc), _P, _P, C.c_int32,
                                C.POINTER(_P)], C.c_int),
    "qltg_ctrct_plan_result": ([_P, C.POINTER(C.c_int32), _I64P, _I64P], C.c_int),
    "qltg_ctrct_plan_result_blocks": ([_P, _P, _P], C.c_int),
    "qltg_ctrct_plan_tasks": ([_P, _I64P, _P], C.c_int),
    "qltg_ctrct_plan_stats": ([_P, C.POINTER(C.c_double), C.POINTER(C.c_double)], C.c_int),
    "qltg_ctrct_exec": ([_P, _P, _P, _P, C.c_int32, _P], C.c_int),
    "qltg_ctrct_exec_stage": ([_P, _P, _P, _P, C.c_int32, C.c_int32, _P], C.c_int),
    "qltg_ctrct_plan_device_status": ([_P, _P], C.c_int),
    "qltg_ctrct_plan_destroy": ([_P], C.c_int),
    "qltg_ctrct_plan_create_contiguous": ([_P, C.POINTER(TensorDesc), C.POINTER(TensorDesc), C.c_int64,
                                           C.c_int64, C.c_int32, C.c_int32, C.c_int32, C.POINTER(_P)], C.c_int),
    "qltg_accum_plan_create": ([_P, C.POINTER(TensorDesc), C.POINTER(TensorDesc), C.c_int64, C.c_int64,
                                C.c_int32, _P, C.c_int32, C.POINTER(_P), C.POINTER(C.c_int32)], C.c_int),
    "qltg_accum_plan_result": ([_P, C.POINTER(C.c_int32), _I64P, _I64P], C.c_int),
    "qltg_accum_plan_result_blocks": ([_P, _P, _P], C.c_int),
    "qltg_accum_exec": ([_P, _P, _P, _P, _P, _P, _P, C.c_int32, _P], C.c_int),
    "qltg_accum_plan_device_status": ([_P, _P], C.c_int),
    "qltg_accum_plan_destroy": ([_P], C.c_int),
    "qltg_axis_diagonal": ([_P, C.POINTER(TensorDesc), C.c_int32, _P, _P, _P, _P, _P, _P], C.c_int),
    "qltg_axis_sector_scalars": ([_P, C.POINTER(TensorDesc), C.c_int32, _P, _P, _P, _P], C.c_int),
    "qltg_axis_rank2_plan_create": ([_P, C.POINTER(TensorDesc), C.POINTER(TensorDesc), C.c_int32, C.POINTER(_P)],
                                    C.c_int),
    "qltg_axis_two_rank2_plan_create": ([_P, C.POINTER(TensorDesc), C.POINTER(TensorDesc), C.c_int32,
                                        C.POINTER(TensorDesc), C.c_int32, C.POINTER(_P)], C.c_int),
    "qltg_axis_monomial_plan_create": ([_P, C.POINTER(TensorDesc), C.c_int32, C.c_int32, _P, _P, _P, C.c_int64, _P,
                                        _P, C.POINTER(_P)], C.c_int),
    "qltg_axis_monomial_exec": ([_P, _P, _P, _P, _P, _P], C.c_int),
    "qltg_axis_project_plan_create": ([_P, C.POINTER(TensorDesc), C.c_int32, _P, _P, C.POINTER(_P)], C.c_int),
    "qltg_lincomb_plan_create": ([_P, C.c_int32, _P, _P, _P, _P, C.c_int32, C.POINTER(_P)], C.c_int),
    "qltg_lincomb_plan_result": ([_P, C.POINTER(C.c_int32), _I64P, _I64P], C.c_int),
    "qltg_lincomb_plan_result_blocks": ([_P, _P, _P], C.c_int),
    "qltg_lincomb_exec": ([_P, _P, _P, _P, _P], C.c_int),
    "qltg_lincomb_plan_destroy": ([_P], C.c_int),
    "qltg_axis_plan_result": ([_P, C.POINTER(C.c_int32), _I64P, _I64P], C.c_int),
    "qltg_axis_plan_result_blocks": ([_P, _P, _P], C.c_int),
    "qltg_axis_plan_exec": ([_P, _P, _P, _P, _P, C.c_int32, _P], C.c_int),
    "qltg_axis_plan_device_status": ([_P, _P], C.c_int),
    "qltg_axis_plan_destroy": ([_P], C.c_int),
    "qltg_qlten_open": ([C.c_char_p, C.c_int32, C.c_int32, C.c_int32, C.POINTER(_P)], C.c_int),
    "qltg_qlten_info": ([_P, C.POINTER(C.c_int32), _I64P, _I64P, _I64P], C.c_int),
    "qltg_qlten_meta": ([_P, _P, _P, _P, _P, _P], C.c_int),
    "qltg_qlten_read_data": ([_P, _P, C.c_int32, _P], C.c_int),
    "qltg_qlten_close": ([_P], C.c_int),
    "qltg_qlten_write": ([C.c_char_p, C.POINTER(TensorDesc), _P, C.c_int32, _P], C.c_int),
    "qltg_ctrct_plan_set_schedule": ([_P, C.c_int32, C.c_int32, _P], C.c_int),
    "qltg_ctrct_plan_get_schedule": ([_P, C.POINTER(C.c_int32), C.POINTER(C.c_int32), _P, _P], C.c_int),
    "qltg_ctrct_plan_tune": ([_P, _P, _P, _P, C.c_int32, _P, C.POINTER(C.c_int32)], C.c_int),
    "qltg_ctrct_plan_split_stats": ([_P, _I64P, C.POINTER(C.c_double)], C.c_int),
    "qltg_matvec_mpo_form": ([_P, C.POINTER(C.c_int32), C.POINTER(C.c_int32), _P], C.c_int),
    "qltg_matvec_set_mpo_form": ([_P, C.c_int32, _P], C.c_int),
    "qltg_matvec_schedule": ([_P, C.c_int32, C.POINTER(C.c_int32), C.POINTER(C.c_int32), _P, _P, _I64P,
                              C.POINTER(C.c_double)], C.c_int),
    "qltg_transpose": ([_P, C.POINTER(TensorDesc), _P, _P, _P, _P], C.c_int),
    "qltg_transpose_noalloc": ([_P, C.POINTER(TensorDesc), _P, _P, _P, _P], C.c_int),
    "qltg_transpose_plan_create": ([_P, C.POINTER(TensorDesc), _P, _P, C.POINTER(_P)], C.c_int),
    "qltg_transpose_plan_exec": ([_P, _P, _P, _P], C.c_int),
    "qltg_transpose_plan_destroy": ([_P], C.c_int),
    "qltg_matvec_create": ([_P, C.POINTER(TensorDesc), _P, C.POINTER(TensorDesc), C.POINTER(TensorDesc), _P,
                            C.POINTER(TensorDesc), _P, C.POINTER(TensorDesc), _P, C.c_int32, _P,
                            C.POINTER(_P)], C.c_int),
    "qltg_matvec_result": ([_P, _I64P, _I64P], C.c_int),
    "qltg_matvec_result_blocks": ([_P, _P, _P], C.c_int),
    "qltg_matvec_stats": ([_P, C.POINTER(C.c_double), _I64P], C.c_int),
    "qltg_matvec_apply": ([_P, _P, _P, _P], C.c_int),
    "qltg_matvec_apply_host": ([_P, _P, _P, _P], C.c_int),
    "qltg_selftest_bounded_wait": ([_P, C.c_int64, _P], C.c_int),
    "qltg_selftest_fp64_rates": ([_P, C.POINTER(C.c_double), C.POINTER(C.c_double), _P], C.c_int),
    "qltg_matvec_device_status": ([_P, _P], C.c_int),
    "qltg_matvec_destroy": ([_P], C.c_int),
    "qltg_lanczos_create": ([_P, C.c_int32, C.POINTER(_P)], C.c_int),
    "qltg_lanczos_start": ([_P, _P, _P], C.c_int),
    "qltg_lanczos_step": ([_P, _P], C.c_int),
    "qltg_lanczos_coeffs": ([_P, C.POINTER(C.c_int32), _P, _P, _P], C.c_int),
    "qltg_lanczos_vector": ([_P, C.c_int32, C.POINTER(_P)], C.c_int),
    "qltg_lanczos_destroy": ([_P], C.c_int),
    "qltg_svd": ([_P, C.POINTER(TensorDesc), _P, C.c_int32, _P, C.c_double, C.c_int64, C.c_int64, _P,
                  C.POINTER(_P)], C.c_int),
    "qltg_qr": ([_P, C.POINTER(TensorDesc), _P, C.c_int32, _P, _P, C.POINTER(_P)], C.c_int),
    "qltg_decomp_info": ([_P, C.POINTER(C.c_double), _I64P], C.c_int),
    "qltg_decomp_tensor_info": ([_P, C.c_int32, _P], C.c_int),
    "qltg_decomp_tensor_export": ([_P, C.c_int32, _P, _P, _P, _P, _P, _P, C.POINTER(_P)], C.c_int),
    "qltg_decomp_destroy": ([_P], C.c_int),
}


def declared_symbols() -> list:
    """Every entry point declared in include/qltg.h."""
    with open(HEADER) as f:
        txt = f.read()
    return sorted(set(re.findall(r"QLTG_API\s+[\w\s\*]+?\b(qltg_\w+)\s*\(", txt)))


class QltgError(RuntimeError):
    def __init__(self, code: int, msg: str):
        super().__init__(f"qltg error {code}: {msg}")
        self.code = code


class EmptySVDResultError(QltgError):
    """Mirror of qlten::EmptySVDResultError (reference framework/exceptions.h)."""


class ContractAccumulateLayoutMismatch(QltgError):
    """Mirror of qlten::detail::ContractAccumulateLayoutMismatch (reference
    tensor_manipulation/contract_contiguous_axes.h:84-88)."""


_lib = None


def lib():
    global _lib
    if _lib is None:
        L = _native.load_qltg()
        for name, (args, res) in _SIGS.items():
            f = getattr(L, name)
            f.argtypes = args
            f.restype = res
        _lib = L
    return _lib


def check(code: int) -> None:
    if code != QLTG_OK:
        msg = lib().qltg_last_error().decode()
        if code == QLTG_ERR_EMPTY_SVD:
            raise EmptySVDResultError(code, msg)
        if code == QLTG_ERR_LAYOUT:
            raise ContractAccumulateLayoutMismatch(code, msg)
        raise QltgError(code, msg)
