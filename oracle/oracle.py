"""ctypes front of the CPU restatement in oracle/oracle.cc.

Test infrastructure only: imported by tests/, by `__graft_entry__.smoke()` to check its result
and by bench.py's CPU-baseline / reference arm. The GPU library never imports it.
The restatement's parity with the reference is pinned by the committed fixtures in
tests/golden/ (produced by the reference itself, see oracle/ref/ref_driver.cc).
"""
from __future__ import annotations

import ctypes as C
import glob
import os
import subprocess
from typing import List, Optional, Sequence

import numpy as np

from tensortoolkit_gb300.tensor import BSTensor

_HERE = os.path.dirname(os.path.abspath(__file__))
_SO = os.path.join(_HERE, "liboracle.so")


class _TensorIn(C.Structure):
    _fields_ = [("rank", C.c_int32), ("ncomp", C.c_int32), ("parity_comp", C.c_int32),
                ("is_complex", C.c_int32), ("dirs", C.c_void_p), ("nsct", C.c_void_p),
                ("qns", C.c_void_p), ("dims", C.c_void_p), ("nblk", C.c_int64),
                ("coords", C.c_void_p), ("data", C.c_void_p)]


_SYNTH = os.path.join(os.path.dirname(_HERE), "tensortoolkit_gb300", "csrc")


def build(force: bool = False) -> str:
    """Compile liboracle.so with g++ (OpenMP, position independent): the restatement plus the
    deterministic workload generator (csrc/synth_capi.cc), so a CPU-only run (the reference
    arm of bench.py) maps no library of the GPU package."""
    srcs = [os.path.join(_HERE, "oracle.cc"), os.path.join(_SYNTH, "synth_capi.cc")]
    deps = srcs + [os.path.join(_SYNTH, "synth.h")]
    if force or not os.path.exists(_SO) or any(os.path.getmtime(_SO) < os.path.getmtime(d) for d in deps):
        subprocess.check_call(["g++", "-O2", "-std=c++17", "-fopenmp", "-fPIC", "-shared", *srcs,
                               "-o", _SO, "-ldl"])
    return _SO


def workload(kind: str, *params: float) -> List[BSTensor]:
    """A named synthetic workload (tensortoolkit_gb300.workloads.generate) made by the copy of
    the generator compiled into liboracle.so: the same bytes as the GPU package's generator."""
    from tensortoolkit_gb300 import workloads
    return workloads.generate(kind, *params, lib=lib())


def find_openblas() -> Optional[str]:
    """SciPy's LP64 OpenBLAS, else NumPy's ILP64 one."""
    cands = []
    try:
        import scipy
        d = os.path.dirname(scipy.__file__) + ".libs"
        cands += sorted(glob.glob(os.path.join(d, "libscipy_openblas-*.so")))
        cands += sorted(glob.glob(os.path.join(d, "libscipy_openblas*.so")))
    except ImportError:
        pass
    d = os.path.dirname(np.__file__) + ".libs"
    cands += sorted(glob.glob(os.path.join(d, "libscipy_openblas64_*.so")))
    cands += sorted(glob.glob(os.path.join(d, "libopenblas*.so*")))
    return cands[0] if cands else None


_lib = None


def lib():
    global _lib
    if _lib is None:
        build()
        L = C.CDLL(_SO)
        L.orc_last_error.restype = C.c_char_p
        L.orc_load_blas.argtypes = [C.c_char_p]
        L.orc_contract.restype = C.c_void_p
        L.orc_contract.argtypes = [C.POINTER(_TensorIn), C.POINTER(_TensorIn), C.c_void_p, C.c_void_p, C.c_int]
        L.orc_contract_contiguous.restype = C.c_void_p
        L.orc_contract_contiguous.argtypes = [C.POINTER(_TensorIn), C.POINTER(_TensorIn), C.c_int64, C.c_int64,
                                              C.c_int]
        L.orc_accumulate.restype = C.c_void_p
        L.orc_accumulate.argtypes = [C.POINTER(_TensorIn), C.POINTER(_TensorIn), C.c_int64, C.c_int64, C.c_int,
                                     C.c_void_p, C.c_void_p, C.c_void_p, C.c_int, C.c_void_p]
        L.orc_svd.restype = C.c_void_p
        L.orc_svd.argtypes = [C.POINTER(_TensorIn), C.c_int, C.c_void_p, C.c_double, C.c_int64, C.c_int64]
        L.orc_qr.restype = C.c_void_p
        L.orc_qr.argtypes = [C.POINTER(_TensorIn), C.c_int, C.c_void_p]
        L.orc_free.argtypes = [C.c_void_p]
        L.orc_num_tasks.restype = C.c_int64
        L.orc_num_tasks.argtypes = [C.c_void_p]
        L.orc_tasks.argtypes = [C.c_void_p, C.c_void_p]
        L.orc_scalar.restype = C.c_double
        L.orc_scalar.argtypes = [C.c_void_p, C.c_int]
        L.orc_tensor_info.argtypes = [C.c_void_p, C.c_int, C.c_void_p]
        L.orc_tensor_export.argtypes = [C.c_void_p, C.c_int] + [C.c_void_p] * 7
        L.orc_set_threads.argtypes = [C.c_int]
        blas = find_openblas()
        if blas is None or L.orc_load_blas(blas.encode()) != 0:
            raise RuntimeError(f"oracle: no usable OpenBLAS ({blas}): {L.orc_last_error().decode()}")
        _lib = L
    return _lib


def set_threads(n: int) -> None:
    lib().orc_set_threads(int(n))


class _In:
    """Keeps the numpy arrays alive while the C side reads them."""

    def __init__(self, t: BSTensor):
        self.dirs, self.nsct, self.qns, self.dims = t.meta_arrays()
        self.coords = np.ascontiguousarray(t.coords, dtype=np.int64)
        self.data = t.raw_f64() if t.size else np.zeros(1)
        p = lambda a: a.ctypes.data if a.size else None
        self.s = _TensorIn(t.rank, t.ncomp, t.parity_comp, int(t.is_complex), p(self.dirs), p(self.nsct),
                           p(self.qns), p(self.dims), t.nblk if t.rank else 0, p(self.coords), p(self.data))


def _export(L, r, i: int) -> BSTensor:
    info = np.zeros(7, np.int64)
    L.orc_tensor_info(r, i, info.ctypes.data)
    rank, ncomp, pc, cplx, nblk, size, ts = (int(x) for x in info)
    dirs = np.zeros(max(rank, 1), np.int32)
    nsct = np.zeros(max(rank, 1), np.int32)
    qns = np.zeros(max(ts * ncomp, 1), np.int32)
    dims = np.zeros(max(ts, 1), np.int64)
    coords = np.zeros(max(nblk * rank, 1), np.int64)
    offs = np.zeros(max(nblk, 1), np.int64)
    data = np.zeros(max(size * (2 if cplx else 1), 1), np.float64)
    L.orc_tensor_export(r, i, dirs.ctypes.data, nsct.ctypes.data, qns.ctypes.data, dims.ctypes.data,
                        coords.ctypes.data, offs.ctypes.data, data.ctypes.data)
    data = data[:size * (2 if cplx else 1)]
    return BSTensor.from_arrays(dirs[:rank], nsct[:rank], qns[:ts * ncomp], dims[:ts], ncomp, pc,
                                coords[:nblk * rank], data, bool(cplx),
                                offsets=offs[:nblk] if rank else None)


def contract(a: BSTensor, b: BSTensor, axes: Sequence[Sequence[int]]):
    """Reference-semantics Contract(a, b, axes) -> (C, tasks[n, 8])."""
    L = lib()
    ia, ib = _In(a), _In(b)
    axa = np.asarray(axes[0], np.int64)
    axb = np.asarray(axes[1], np.int64)
    r = L.orc_contract(C.byref(ia.s), C.byref(ib.s), axa.ctypes.data, axb.ctypes.data, len(axa))
    if not r:
        raise RuntimeError(L.orc_last_error().decode())
    try:
        c = _export(L, r, 0)
        nt = L.orc_num_tasks(r)
        tasks = np.zeros((nt, 8), np.int64)
        if nt:
            L.orc_tasks(r, tasks.ctypes.data)
        return c, tasks
    finally:
        L.orc_free(r)


def contract_contiguous(a: BSTensor, b: BSTensor, a_start: int, b_start: int, n: int) -> BSTensor:
    """Reference-semantics ContractContiguousAxes(a, b, a_start, b_start, n): contracted axes
    (start + i) mod rank, C legs = the saved legs of A then of B, each cyclic from the end of
    its contracted range."""
    L = lib()
    ia, ib = _In(a), _In(b)
    r = L.orc_contract_contiguous(C.byref(ia.s), C.byref(ib.s), int(a_start), int(b_start), int(n))
    if not r:
        raise RuntimeError(L.orc_last_error().decode())
    try:
        return _export(L, r, 0)
    finally:
        L.orc_free(r)


def accumulate(a: BSTensor, b: BSTensor, a_start: int, b_start: int, n: int, alpha, beta,
               c: Optional[BSTensor] = None, allow_expand: bool = True):
    """Reference-semantics ContractTailHeadContiguousAccumulate (allow_expand) /
    TryContractTailHeadContiguousAccumulate: (True, beta c + alpha a.b over the union
    topology), or (False, None) when the layout does not fit."""
    L = lib()
    ia, ib = _In(a), _In(b)
    ic = _In(c) if c is not None else None
    al = np.array([complex(alpha).real, complex(alpha).imag])
    be = np.array([complex(beta).real, complex(beta).imag])
    st = np.zeros(1, np.int32)
    r = L.orc_accumulate(C.byref(ia.s), C.byref(ib.s), int(a_start), int(b_start), int(n), al.ctypes.data,
                         be.ctypes.data, C.byref(ic.s) if ic is not None else None, int(allow_expand),
                         st.ctypes.data)
    if not r:
        if st[0] == 1:
            return False, None
        raise RuntimeError(L.orc_last_error().decode())
    try:
        return True, _export(L, r, 0)
    finally:
        L.orc_free(r)


class EmptySVDResultError(RuntimeError):
    pass


def svd(t: BSTensor, ldims: int, lqndiv: Sequence[int], trunc_err: float, dmin: int, dmax: int):
    """Reference-semantics SVD -> (U, S, Vt, actual_trunc_err, D)."""
    L = lib()
    it = _In(t)
    div = np.asarray(lqndiv, np.int32)
    r = L.orc_svd(C.byref(it.s), int(ldims), div.ctypes.data, float(trunc_err), int(dmin), int(dmax))
    if not r:
        msg = L.orc_last_error().decode()
        if "EmptySVDResult" in msg:
            raise EmptySVDResultError(msg)
        raise RuntimeError(msg)
    try:
        return (_export(L, r, 0), _export(L, r, 1), _export(L, r, 2), L.orc_scalar(r, 0),
                int(L.orc_scalar(r, 1)))
    finally:
        L.orc_free(r)


def qr(t: BSTensor, ldims: int, lqndiv: Sequence[int]):
    """Reference-semantics QR -> (Q, R)."""
    L = lib()
    it = _In(t)
    div = np.asarray(lqndiv, np.int32)
    r = L.orc_qr(C.byref(it.s), int(ldims), div.ctypes.data)
    if not r:
        raise RuntimeError(L.orc_last_error().decode())
    try:
        return _export(L, r, 0), _export(L, r, 1)
    finally:
        L.orc_free(r)


def matvec(lenv: BSTensor, psi: BSTensor, mpo1: BSTensor, mpo2: BSTensor, renv: BSTensor):
    """The reference's two-site chain (tests/test_tensor_manipulation/test_ten_ctrct_1sct.cc:253-257)."""
    t1, _ = contract(lenv, psi, ((0,), (0,)))
    t2, _ = contract(t1, mpo1, ((0, 2), (0, 1)))
    t3, _ = contract(t2, mpo2, ((4, 1), (0, 1)))
    out, _ = contract(t3, renv, ((4, 1), (1, 0)))
    return out, (t1, t2, t3)


def read_qtb(path: str) -> dict:
    """Read a QTB1 container written by oracle/qtb_io.h."""
    dt = {0: np.float64, 1: np.int64, 2: np.int32, 3: np.uint8}
    out = {}
    with open(path, "rb") as f:
        buf = f.read()
    assert buf[:4] == b"QTB1"
    p = 4
    while p < len(buf):
        nl = int(np.frombuffer(buf, np.uint32, 1, p)[0]); p += 4
        name = buf[p:p + nl].decode(); p += nl
        code = buf[p]; p += 1
        nd = int(np.frombuffer(buf, np.uint32, 1, p)[0]); p += 4
        shape = tuple(int(x) for x in np.frombuffer(buf, np.uint64, nd, p)); p += 8 * nd
        n = int(np.prod(shape, dtype=np.int64)) if nd else 1
        t = dt[code]
        nb = n * np.dtype(t).itemsize
        out[name] = np.frombuffer(buf, t, n, p).reshape(shape).copy(); p += nb
    return out
