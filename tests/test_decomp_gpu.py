"""Parity of the batched block SVD (one-sided Jacobi) and QR (Householder) with the
reference (golden fixtures) and the CPU restatement (full-size cases), through the C ABI.

Bar: U / S / Vt and Q / R block topology bit-exact (legs, mid-leg sectors, blocks,
offsets); same kept dimension D; singular values within 1e-10; truncation error within
1e-12. Singular vectors are compared gauge-invariantly (each kept pair (u_i, v_i) is
fixed only up to a phase): |<u_mine, u_ref>| = 1 for non-degenerate values, and
U S Vt reproduces the reference's U S Vt. QR follows LAPACK's reflector convention, so
Q and R are compared directly."""
import numpy as np
import pytest

from oracle import oracle
from tensortoolkit_gb300 import workloads
from tensortoolkit_gb300.api import QR, SVD, DTensor
from tensortoolkit_gb300.capi import EmptySVDResultError
from tensortoolkit_gb300.tensor import BSTensor, rel_frob, same_topology
from tests.svd_check import check_svd

pytestmark = pytest.mark.gpu

SVD_CASES = ["svd_u1_full", "svd_u1_trunc", "svd_u1_dmax", "svd_u1_dmin", "svd_stress_small", "svd_f"]


@pytest.mark.parametrize("case", SVD_CASES)
def test_svd_golden(gpu, golden, case):
    rec = golden(case)
    t = BSTensor.from_record(rec, "T")
    ldims = int(rec["ldims"][0])
    u, s, vt, err, D = SVD(DTensor.from_host(t), ldims, [0] * t.ncomp, float(rec["trunc"][0]),
                           int(rec["Dmin"][0]), int(rec["Dmax"][0]))
    check_svd(t, u.to_host(), s.to_host(), vt.to_host(), err, D, BSTensor.from_record(rec, "U"),
              BSTensor.from_record(rec, "S"), BSTensor.from_record(rec, "Vt"), float(rec["err"][0]),
              int(rec["D"][0]), ldims)


@pytest.mark.parametrize("case", ["qr_u1", "qr_f"])
def test_qr_golden(gpu, golden, case):
    rec = golden(case)
    t = BSTensor.from_record(rec, "T")
    q, r = QR(DTensor.from_host(t), int(rec["ldims"][0]), [0] * t.ncomp)
    for mine, name in ((q.to_host(), "Q"), (r.to_host(), "R")):
        ref = BSTensor.from_record(rec, name)
        assert same_topology(mine, ref), name
        assert rel_frob(mine.data, ref.data) <= 1e-12, (name, rel_frob(mine.data, ref.data))


@pytest.mark.parametrize("D,trunc,dmax", [(2000, 1e-9, 2000), (2000, 1e-4, 600)])
def test_svd_spectrum_psi_vs_oracle(gpu, D, trunc, dmax):
    """Config 3: the D=2000 two-site psi with a controlled spectrum s_j = exp(-0.01 j)."""
    t = workloads.svd_psi(D, 20, 6.0, 3)
    ru, rs, rvt, rerr, rD = oracle.svd(t, 2, [0], trunc, 1, dmax)
    u, s, vt, err, Dk = SVD(DTensor.from_host(t), 2, [0], trunc, 1, dmax)
    check_svd(t, u.to_host(), s.to_host(), vt.to_host(), err, Dk, ru, rs, rvt, rerr, rD, 2)


def test_svd_stress_vs_oracle(gpu):
    """41 square block-matrices with sizes 10..800 (rank-2 tensor), same spectrum rule."""
    t = workloads.svd_stress(41, 10, 800, 3)
    ru, rs, rvt, rerr, rD = oracle.svd(t, 1, [0], 1e-9, 1, 100000)
    u, s, vt, err, Dk = SVD(DTensor.from_host(t), 1, [0], 1e-9, 1, 100000)
    check_svd(t, u.to_host(), s.to_host(), vt.to_host(), err, Dk, ru, rs, rvt, rerr, rD, 1)


@pytest.mark.parametrize("D,trunc,dmax", [(1200, 1e-12, 100000), (3000, 1e-8, 2000)])
def test_svd_complex_fermionic_vs_oracle(gpu, D, trunc, dmax):
    """The complex128 fU(1) x U(1) psi of the Hubbard workload (5544 blocks, a thousand and
    more block-matrices): the complex Jacobi path, whole and cut at Dmax."""
    _, psi, *_ = workloads.hubbard(D)
    div = [0] * psi.ncomp
    ru, rs, rvt, rerr, rD = oracle.svd(psi, 2, div, trunc, 1, dmax)
    u, s, vt, err, Dk = SVD(DTensor.from_host(psi), 2, div, trunc, 1, dmax)
    check_svd(psi, u.to_host(), s.to_host(), vt.to_host(), err, Dk, ru, rs, rvt, rerr, rD, 2)


def test_qr_complex_fermionic_vs_oracle(gpu):
    """Complex Householder (LAPACK's zlarfg convention: real diagonal of R), so Q and R
    compare directly."""
    _, psi, *_ = workloads.hubbard(3000)
    div = [0] * psi.ncomp
    rq, rr = oracle.qr(psi, 2, div)
    q, r = QR(DTensor.from_host(psi), 2, div)
    q, r = q.to_host(), r.to_host()
    assert same_topology(q, rq) and same_topology(r, rr)
    assert rel_frob(q.data, rq.data) <= 1e-11
    assert rel_frob(r.data, rr.data) <= 1e-11


def test_qr_psi_vs_oracle(gpu):
    lenv, psi, *_ = workloads.heisenberg(2000, 20, 6.0, 5)
    rq, rr = oracle.qr(psi, 2, [0])
    q, r = QR(DTensor.from_host(psi), 2, [0])
    q, r = q.to_host(), r.to_host()
    assert same_topology(q, rq) and same_topology(r, rr)
    assert rel_frob(q.data, rq.data) <= 1e-11
    assert rel_frob(r.data, rr.data) <= 1e-11


def test_empty_svd_raises(gpu, golden):
    # reference tests/test_tensor_manipulation/test_ten_svd.cc:699-711
    rec = golden("svd_u1_full")
    t = BSTensor.from_record(rec, "T")
    empty = BSTensor(t.legs, np.zeros((0, t.rank), np.int64), np.float64, np.zeros(0))
    with pytest.raises(EmptySVDResultError):
        SVD(DTensor.from_host(empty), 2, [0], 0.0, 1, 100)
