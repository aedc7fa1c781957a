"""Pin the CPU restatement of ContractContiguousAxes and of the accumulate forms
(ContractTailHeadContiguousAccumulate / TryContractTailHeadContiguousAccumulate) to the
reference's own outputs (tests/golden/ctrct_contig.npz, made by the reference driver).

Cases (U(1) real "u_", fermionic U(1)xU(1) complex "f_"):
  hh, wrap, mid, tt, ht   ContractContiguousAxes over head/tail, wrapped ({3, 0}) and middle
                          ({1, 2}: saved legs come out as 3, 0) ranges, all four side pairs
  acc_default             default output, beta = 0
  acc_same                output with the contraction's own topology
  acc_expand              output holding only other blocks: union topology
  acc_superset            output with extra blocks: scaled by beta, no expansion
  try_fail / try_ok       the no-expansion probe refuses / accepts
"""
import numpy as np
import pytest

from oracle import oracle
from tensortoolkit_gb300.tensor import BSTensor, rel_frob, same_topology

CONTIG = ["hh", "wrap", "mid", "tt", "ht"]
ACCUM = ["acc_default", "acc_same", "acc_expand", "acc_superset"]
TRY = ["try_fail", "try_ok"]


def _params(rec, tag):
    a0, b0, n, a_tail, b_head = (int(x) for x in rec[tag + ".params"])
    return a0, b0, n, bool(a_tail), bool(b_head)


def _scalars(rec, tag):
    al, be = rec[tag + ".alpha"], rec[tag + ".beta"]
    return complex(al[0], al[1]), complex(be[0], be[1])


def _cplx_or_real(x: complex, t: BSTensor):
    return x if t.is_complex else x.real


@pytest.mark.parametrize("pre", ["u_", "f_"])
@pytest.mark.parametrize("case", CONTIG)
def test_contiguous_matches_reference(golden, pre, case):
    rec = golden("ctrct_contig")
    tag = pre + case
    a = BSTensor.from_record(rec, tag + ".A")
    b = BSTensor.from_record(rec, tag + ".B")
    ref = BSTensor.from_record(rec, tag + ".C")
    a0, b0, n, _, _ = _params(rec, tag)
    c = oracle.contract_contiguous(a, b, a0, b0, n)
    assert same_topology(c, ref)
    assert rel_frob(c.data, ref.data) <= 1e-13


@pytest.mark.parametrize("pre", ["u_", "f_"])
@pytest.mark.parametrize("case", ACCUM + TRY)
def test_accumulate_matches_reference(golden, pre, case):
    rec = golden("ctrct_contig")
    tag = pre + case
    a = BSTensor.from_record(rec, tag + ".A")
    b = BSTensor.from_record(rec, tag + ".B")
    ref = BSTensor.from_record(rec, tag + ".C")
    c0 = BSTensor.from_record(rec, tag + ".C0") if tag + ".C0.dirs" in rec else None
    a0, b0, n, _, _ = _params(rec, tag)
    al, be = _scalars(rec, tag)
    ok, c = oracle.accumulate(a, b, a0, b0, n, _cplx_or_real(al, a), _cplx_or_real(be, a), c0,
                              allow_expand=case not in TRY)
    if case in TRY:
        assert ok == bool(int(rec[tag + ".ok"][0]))
        if not ok:   # the reference left the output unchanged
            assert same_topology(ref, c0) and np.array_equal(ref.data, c0.data)
            return
    assert ok
    assert same_topology(c, ref)
    assert rel_frob(c.data, ref.data) <= 1e-13


def test_cases_exercise_the_semantics(golden):
    rec = golden("ctrct_contig")
    # the middle range reorders saved legs: C's first leg is A's leg 3
    a = BSTensor.from_record(rec, "u_mid.A")
    c = BSTensor.from_record(rec, "u_mid.C")
    assert c.legs[0].same_space(a.legs[3]) and c.legs[1].same_space(a.legs[0])
    # expansion grew the output; the superset case kept its topology
    for pre in ("u_", "f_"):
        c0 = BSTensor.from_record(rec, pre + "acc_expand.C0")
        c1 = BSTensor.from_record(rec, pre + "acc_expand.C")
        assert c1.nblk > c0.nblk
        s0 = BSTensor.from_record(rec, pre + "acc_superset.C0")
        s1 = BSTensor.from_record(rec, pre + "acc_superset.C")
        assert same_topology(s0, s1)
