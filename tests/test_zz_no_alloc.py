"""The allocation-free permute entry point, qltg_transpose_noalloc.

Callers that cannot allocate device memory while they run - a sweep whose device memory
was handed up front to another framework's pool, where a cudaMalloc fails or evicts that
pool's cache, or a loop that cannot pay for the device-wide synchronisation of cudaMalloc /
cudaFree - use this variant. Instead of a fresh device work list per call, it writes the
per-block permutation descriptors into a fixed table compiled into the library (at most
4096 blocks). These tests call it through the C ABI and require bit for bit the result of
qltg_transpose (a permutation with exact sign flips: no rounding is involved), on two calls
in a row that reuse the shared table, and a clean error beyond the table's size.

This file is collected last on purpose, so a run that stops at the first failure has run
every other test already; it also passes on its own in a fresh process."""
import ctypes as C

import numpy as np
import pytest
import torch

from tensortoolkit_gb300 import capi, workloads
from tensortoolkit_gb300.api import DTensor, _Desc, context, stream_ptr

pytestmark = pytest.mark.gpu


def _run(fn, t: DTensor, perm):
    out = torch.zeros_like(t.buf)
    d = _Desc(t.meta)
    p = np.asarray(perm, np.int32)
    rc = fn(context(0).h, d.ref, C.c_void_p(t.ptr), p.ctypes.data, C.c_void_p(out.data_ptr()), stream_ptr(0))
    return rc, out


def test_noalloc_matches_transpose_twice(gpu):
    L = capi.lib()
    # first call: fermionic complex psi (exercises the block signs); second call: a real
    # U(1) environment with a different rank and permutation, overwriting the shared table
    _, psi_f, *_ = workloads.hubbard(400, 4, 9)
    lenv, *_ = workloads.heisenberg(1200, 12, 4.0, 1)
    for host, perm in ((psi_f, (3, 0, 2, 1)), (lenv, (2, 0, 1))):
        t = DTensor.from_host(host)
        rc_ref, ref = _run(L.qltg_transpose, t, perm)
        assert rc_ref == capi.QLTG_OK, L.qltg_last_error()
        rc, out = _run(L.qltg_transpose_noalloc, t, perm)
        assert rc == capi.QLTG_OK, L.qltg_last_error()
        torch.cuda.synchronize()
        assert np.array_equal(out.cpu().numpy(), ref.cpu().numpy())


def test_noalloc_rejects_more_blocks_than_its_table(gpu):
    L = capi.lib()
    _, psi, *_ = workloads.hubbard(800, 10, 4)     # 400 bond sectors: more than 4096 blocks
    assert psi.nblk > 4096
    rc, _ = _run(L.qltg_transpose_noalloc, DTensor.from_host(psi), (0, 2, 1, 3))
    assert rc == capi.QLTG_ERR_INVALID
    assert b"4096" in L.qltg_last_error()
