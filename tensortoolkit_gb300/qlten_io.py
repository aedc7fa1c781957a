"""`.qlten` stream files (the reference's QLTensor serialisation) for host tensors.

The parsing and writing run in libqltg.so (`qltg_qlten_*`, include/qltg.h); these wrappers
move host buffers. Device-direct forms (`read_qlten` / `write_qlten` on DTensors) are in
`tensortoolkit_gb300.api`.

Quantum number types (they are not recorded in the file; every stored hash is checked, so a
wrong type is rejected): "U1QN", "U1U1QN", "fU1U1QN" (fermion parity = first component).
"""
from __future__ import annotations

import ctypes as C
from typing import Tuple

import numpy as np

from . import capi
from .capi import check, lib
from .tensor import BSTensor

QN_TYPES = {"U1QN": (1, -1), "U1U1QN": (2, -1), "fU1U1QN": (2, 0)}
DTYPES = {"f64": capi.QLTG_F64, "c128": capi.QLTG_C128}


class QltenFile:
    """An opened .qlten file: header parsed, raw buffer not read yet."""

    def __init__(self, path: str, qn: str = "U1QN", dtype: str = "f64"):
        ncomp, pc = QN_TYPES[qn]
        self.h = None
        h = C.c_void_p()
        check(lib().qltg_qlten_open(path.encode(), ncomp, pc, DTYPES[dtype], C.byref(h)))
        self.h = h
        rank, ts, nblk, size = C.c_int32(), C.c_int64(), C.c_int64(), C.c_int64()
        check(lib().qltg_qlten_info(h, C.byref(rank), C.byref(ts), C.byref(nblk), C.byref(size)))
        r, nb = rank.value, nblk.value
        dirs = np.zeros(max(r, 1), np.int32)
        nsct = np.zeros(max(r, 1), np.int32)
        qns = np.zeros(max(ts.value * ncomp, 1), np.int32)
        dims = np.zeros(max(ts.value, 1), np.int64)
        coords = np.zeros(max(nb * r, 1), np.int64)
        check(lib().qltg_qlten_meta(h, dirs.ctypes.data, nsct.ctypes.data, qns.ctypes.data, dims.ctypes.data,
                                    coords.ctypes.data))
        self.size = size.value
        self.is_complex = dtype == "c128"
        self.meta = BSTensor.from_arrays(dirs[:r], nsct[:r], qns[: ts.value * ncomp], dims[: ts.value], ncomp, pc,
                                         coords[: nb * r], np.zeros(self.size * (2 if self.is_complex else 1)),
                                         self.is_complex)

    def read_host(self) -> BSTensor:
        raw = np.zeros(max(self.size * (2 if self.is_complex else 1), 1), np.float64)
        check(lib().qltg_qlten_read_data(self.h, raw.ctypes.data, 0, None))
        t = self.meta.copy()
        data = raw[: self.size * (2 if self.is_complex else 1)]
        t.data = data.view(np.complex128).copy() if self.is_complex else data.copy()
        return t

    def close(self) -> None:
        if self.h:
            lib().qltg_qlten_close(self.h)
            self.h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass


def read_qlten_host(path: str, qn: str = "U1QN", dtype: str = "f64") -> BSTensor:
    """Read a .qlten file into a host tensor (the reference's operator>> on a QLTensor)."""
    f = QltenFile(path, qn, dtype)
    try:
        return f.read_host()
    finally:
        f.close()


def _desc(t: BSTensor) -> Tuple[capi.TensorDesc, tuple]:
    dirs, nsct, qns, dims = t.meta_arrays()
    coords = np.ascontiguousarray(t.coords.reshape(-1), dtype=np.int64)
    p = lambda a: a.ctypes.data if a.size else None
    d = capi.TensorDesc(t.rank, capi.QLTG_C128 if t.is_complex else capi.QLTG_F64, t.ncomp, t.parity_comp, p(dirs),
                        p(nsct), p(qns), p(dims), t.nblk if t.rank else (1 if t.size else 0), p(coords))
    return d, (dirs, nsct, qns, dims, coords)


def write_qlten_host(path: str, t: BSTensor) -> None:
    """Write a host tensor as a .qlten file (the reference's operator<< on a QLTensor)."""
    d, keep = _desc(t)
    raw = t.raw_f64() if t.size else np.zeros(1)
    check(lib().qltg_qlten_write(path.encode(), C.byref(d), raw.ctypes.data, 0, None))
    del keep
