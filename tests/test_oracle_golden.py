"""Pin the CPU restatement (oracle/oracle.cc) to the reference's own outputs.

The fixtures in tests/golden/ were produced by the reference implementation (its CPU
Contract / SVD / QR, compiled from its sources; see tests/golden/make_golden.py). Every
case here runs the restatement on the same inputs and requires identical block topology,
task lists and fermion signs, and values equal to rounding."""
import numpy as np
import pytest

from oracle import oracle
from tensortoolkit_gb300.tensor import BSTensor, rel_frob, same_topology
from tests.svd_check import check_svd

CTRCT_CASES = [
    ("cfg1", ["c"]),
    ("matvec_u1_small", ["s1", "s2", "s3", "s4"]),
    ("matvec_f_small", ["s1", "s2", "s3", "s4"]),
    ("ctrct_misc_u1", ["u_scalar", "u_perm", "u_mid", "f_scalar", "f_in", "f_rev", "f_env", "f_mpo"]),
]


def _axes(rec, tag, ra):
    ax = rec[tag + ".axes"]
    n = len(ax) // 2
    return [list(ax[:n]), list(ax[n:])]


@pytest.mark.parametrize("case,tags", CTRCT_CASES)
def test_contract_matches_reference(golden, case, tags):
    rec = golden(case)
    for tag in tags:
        a = BSTensor.from_record(rec, tag + ".A")
        b = BSTensor.from_record(rec, tag + ".B")
        ref_c = BSTensor.from_record(rec, tag + ".C")
        c, tasks = oracle.contract(a, b, _axes(rec, tag, a.rank))
        ref_tasks = rec[tag + ".tasks"].reshape(-1, 8)
        assert np.array_equal(tasks, ref_tasks), f"{case}/{tag}: task list differs"
        if ref_c.rank:
            assert same_topology(c, ref_c), f"{case}/{tag}: block topology differs"
        assert c.size == ref_c.size
        assert rel_frob(c.data, ref_c.data) <= 1e-13, f"{case}/{tag}: values differ"


def test_fermion_signs_exercised(golden):
    rec = golden("matvec_f_small")
    signs = np.concatenate([rec[f"s{i}.tasks"].reshape(-1, 8)[:, 6] for i in range(1, 5)])
    assert (signs == -1).any() and (signs == 1).any()
    rec = golden("ctrct_misc_u1")
    assert (rec["f_in.tasks"].reshape(-1, 8)[:, 6] == -1).any()


def test_matvec_chain_matches_reference(golden):
    for case in ("matvec_u1_small", "matvec_f_small"):
        rec = golden(case)
        lenv = BSTensor.from_record(rec, "s1.A")
        psi = BSTensor.from_record(rec, "s1.B")
        mpo1 = BSTensor.from_record(rec, "s2.B")
        mpo2 = BSTensor.from_record(rec, "s3.B")
        renv = BSTensor.from_record(rec, "s4.B")
        out, _ = oracle.matvec(lenv, psi, mpo1, mpo2, renv)
        ref = BSTensor.from_record(rec, "s4.C")
        assert same_topology(out, ref)
        assert rel_frob(out.data, ref.data) <= 1e-13


SVD_CASES = ["svd_u1_full", "svd_u1_trunc", "svd_u1_dmax", "svd_u1_dmin", "svd_stress_small", "svd_f"]


@pytest.mark.parametrize("case", SVD_CASES)
def test_svd_matches_reference(golden, case):
    rec = golden(case)
    t = BSTensor.from_record(rec, "T")
    ldims = int(rec["ldims"][0])
    div = [0] * t.ncomp
    u, s, vt, err, D = oracle.svd(t, ldims, div, float(rec["trunc"][0]), int(rec["Dmin"][0]), int(rec["Dmax"][0]))
    assert D == int(rec["D"][0])
    assert abs(err - float(rec["err"][0])) <= 1e-12
    for mine, name in ((u, "U"), (s, "S"), (vt, "Vt")):
        ref = BSTensor.from_record(rec, name)
        assert same_topology(mine, ref), f"{case}: {name} topology differs"
        # same LAPACK routine on the same dense block-matrices: equal to rounding
        assert rel_frob(mine.data, ref.data) <= 1e-12, f"{case}: {name} values differ"
    # the gauge-invariant SVD check used for the GPU Jacobi SVD accepts the oracle's result
    check_svd(t, u, s, vt, err, D, BSTensor.from_record(rec, "U"), BSTensor.from_record(rec, "S"),
              BSTensor.from_record(rec, "Vt"), float(rec["err"][0]), int(rec["D"][0]), ldims)


@pytest.mark.parametrize("case", ["qr_u1", "qr_f"])
def test_qr_matches_reference(golden, case):
    rec = golden(case)
    t = BSTensor.from_record(rec, "T")
    q, r = oracle.qr(t, int(rec["ldims"][0]), [0] * t.ncomp)
    for mine, name in ((q, "Q"), (r, "R")):
        ref = BSTensor.from_record(rec, name)
        assert same_topology(mine, ref), f"{case}: {name} topology differs"
        assert rel_frob(mine.data, ref.data) <= 1e-12


def test_empty_svd_raises(golden):
    # reference tests/test_tensor_manipulation/test_ten_svd.cc:699-711: a tensor with legs but
    # no data blocks throws EmptySVDResultError
    rec = golden("svd_u1_full")
    t = BSTensor.from_record(rec, "T")
    empty = BSTensor(t.legs, np.zeros((0, t.rank), np.int64), np.float64, np.zeros(0))
    with pytest.raises(oracle.EmptySVDResultError):
        oracle.svd(empty, 2, [0], 0.0, 1, 100)
