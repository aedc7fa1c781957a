"""CPU-side checks of the C ABI boundary: the library loads and exports every entry point
declared in include/qltg.h; host-side validation rejects malformed descriptors before any
device work."""
import ctypes as C
import os

import numpy as np
import pytest

from tensortoolkit_gb300 import _native, capi


def test_header_declares_the_boundary():
    syms = capi.declared_symbols()
    for s in ("qltg_create", "qltg_ctrct_plan_create", "qltg_ctrct_exec", "qltg_matvec_create",
              "qltg_matvec_apply", "qltg_svd", "qltg_qr", "qltg_transpose", "qltg_last_error"):
        assert s in syms
    assert set(syms) <= set(capi._SIGS), "ctypes signatures missing for: %s" % (set(syms) - set(capi._SIGS))


def test_library_exports_every_declared_symbol():
    if not os.path.exists(_native.LIB_QLTG):
        _native.build_qltg()
    lib = C.CDLL(_native.LIB_QLTG)
    missing = [s for s in capi.declared_symbols() if not hasattr(lib, s)]
    assert not missing, missing


def test_errors_are_status_codes_not_exits():
    # no GPU needed: a null context is rejected on the host with a message
    L = capi.lib()
    h = C.c_void_p()
    rc = L.qltg_ctrct_plan_create(None, None, None, None, None, 0, C.byref(h))
    assert rc == capi.QLTG_ERR_INVALID
    assert b"null" in L.qltg_last_error()
    rc = L.qltg_matvec_apply(None, None, None, None)
    assert rc == capi.QLTG_ERR_INVALID


def test_create_without_device_fails_cleanly():
    import torch
    if torch.cuda.is_available():
        pytest.skip("a device is present")
    h = C.c_void_p()
    rc = capi.lib().qltg_create(0, C.byref(h))
    assert rc in (capi.QLTG_ERR_CUDA, capi.QLTG_ERR_INVALID)
    assert capi.lib().qltg_last_error()
