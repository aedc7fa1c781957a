"""Synthetic workloads with the shapes of the reference's two-site H*psi, block SVD and
fermionic Hubbard cases, generated deterministically by csrc/synth.h (mt19937_64 +
Box-Muller) so the GPU path, the CPU oracle and the reference driver see identical bytes.

No dataset is involved: the reference's own matvec test reads environment files that are
not in its repository (tests/test_tensor_manipulation/test_ten_ctrct_1sct.cc:147-257), so
seeded synthetic tensors with the same leg structure stand in for them.
"""
from __future__ import annotations

import ctypes as C
from typing import List

import numpy as np

from . import _native
from .tensor import BSTensor


def _lib(L=None):
    """The generator library: libqltg_synth.so, or another library that exports the same
    qltg_synth_* entry points (the CPU oracle compiles the generator into its own library,
    so a CPU-only process never maps this package's shared objects)."""
    if L is None:
        L = _native.load_synth()
    if not getattr(L, "_qltg_synth_typed", False):
        L.qltg_synth_create.restype = C.c_void_p
        L.qltg_synth_create.argtypes = [C.c_char_p, C.c_void_p, C.c_int]
        L.qltg_synth_last_error.restype = C.c_char_p
        L.qltg_synth_count.argtypes = [C.c_void_p]
        L.qltg_synth_info.argtypes = [C.c_void_p, C.c_int, C.c_void_p]
        L.qltg_synth_export.argtypes = [C.c_void_p, C.c_int] + [C.c_void_p] * 7
        L.qltg_synth_free.argtypes = [C.c_void_p]
        L._qltg_synth_typed = True
    return L


def generate(kind: str, *params: float, lib=None) -> List[BSTensor]:
    L = _lib(lib)
    p = np.asarray(params, np.float64)
    h = L.qltg_synth_create(kind.encode(), p.ctypes.data if p.size else None, len(p))
    if not h:
        raise ValueError(L.qltg_synth_last_error().decode())
    try:
        out = []
        for i in range(L.qltg_synth_count(h)):
            info = np.zeros(7, np.int64)
            L.qltg_synth_info(h, i, info.ctypes.data)
            rank, ncomp, pc, cplx, nblk, size, ts = (int(x) for x in info)
            dirs = np.zeros(rank, np.int32)
            nsct = np.zeros(rank, np.int32)
            qns = np.zeros(ts * ncomp, np.int32)
            dims = np.zeros(ts, np.int64)
            coords = np.zeros(nblk * rank, np.int64)
            offs = np.zeros(nblk, np.int64)
            data = np.zeros(size * (2 if cplx else 1), np.float64)
            L.qltg_synth_export(h, i, dirs.ctypes.data, nsct.ctypes.data, qns.ctypes.data,
                                dims.ctypes.data, coords.ctypes.data, offs.ctypes.data, data.ctypes.data)
            out.append(BSTensor.from_arrays(dirs, nsct, qns, dims, ncomp, pc, coords, data, bool(cplx),
                                            offsets=offs))
        return out
    finally:
        L.qltg_synth_free(h)


def config1(seed: int = 0):
    """Rank-3 U(1) A, B (legs 36 x 2 x 38); contract A.leg2 with B.leg0."""
    return generate("cfg1", seed)


def heisenberg(D: int, qmax: int, sigma: float, seed: int = 1, hermitian: bool = False, lib=None):
    """(lenv, psi, mpo1, mpo2, renv) of the U(1) two-site matvec at bond dimension D."""
    return generate("matvec_u1h" if hermitian else "matvec_u1", qmax, sigma, D, seed, lib=lib)


def heisenberg_complex_hermitian(D: int, qmax: int, sigma: float, seed: int = 1):
    """The U(1) two-site matvec in complex128 with a complex-Hermitian effective Hamiltonian
    (environments E(a, w, a') = conj(E(a', wbar, a)), the Heisenberg MPO)."""
    return generate("matvec_u1hc", qmax, sigma, D, seed)


def hubbard(D: int, half: int = 10, seed: int = 4):
    """(lenv, psi, mpo1, mpo2, renv) of the fermionic U(1)xU(1) complex128 matvec."""
    return generate("matvec_f", half, D, seed)


def svd_psi(D: int, qmax: int, sigma: float, seed: int = 3) -> BSTensor:
    return generate("svd_u1", qmax, sigma, D, seed)[0]


def svd_stress(nb: int = 41, lo: int = 10, hi: int = 800, seed: int = 3) -> BSTensor:
    return generate("svd_stress", nb, lo, hi, seed)[0]


# Named benchmark/parity configurations (sizes from the reference's headline cases).
CONFIGS = {
    "heisenberg_d2000": dict(D=2000, qmax=20, sigma=6.0, seed=1),
    "heisenberg_d4000": dict(D=4000, qmax=30, sigma=9.0, seed=1),
    "hubbard_d6000": dict(D=6000, half=10, seed=4),
}
