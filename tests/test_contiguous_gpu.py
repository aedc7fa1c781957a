"""ContractContiguousAxes and the accumulate forms on the GPU, through the C ABI, against the
reference's own outputs (tests/golden/ctrct_contig.npz) and the oracle.

Bar: block topology identical to the reference's; values within 1e-12 relative Frobenius
(FP64 and split precision, real and complex); the no-expansion form refuses exactly when
the reference's does and then leaves C untouched."""
import numpy as np
import pytest

from oracle import oracle
from tensortoolkit_gb300 import capi
from tensortoolkit_gb300.api import (AccumulatePlan, ContiguousContractionPlan, ContractContiguousAxes,
                                     ContractTailHeadContiguousAccumulate, DTensor,
                                     TryContractTailHeadContiguousAccumulate)
from tensortoolkit_gb300.tensor import BSTensor, rel_frob, same_topology

pytestmark = pytest.mark.gpu

TOL = 1e-12
CONTIG = ["hh", "wrap", "mid", "tt", "ht"]
ACCUM = ["acc_default", "acc_same", "acc_expand", "acc_superset"]


def _params(rec, tag):
    a0, b0, n, a_tail, b_head = (int(x) for x in rec[tag + ".params"])
    return a0, b0, n, "tail" if a_tail else "head", "head" if b_head else "tail"


def _scalars(rec, tag, t):
    al, be = rec[tag + ".alpha"], rec[tag + ".beta"]
    al, be = complex(al[0], al[1]), complex(be[0], be[1])
    return (al, be) if t.is_complex else (al.real, be.real)


def _modes(t):
    return ["fp64", "split"]


@pytest.mark.parametrize("pre", ["u_", "f_"])
@pytest.mark.parametrize("case", CONTIG)
def test_contiguous_vs_reference(gpu, golden, pre, case):
    rec = golden("ctrct_contig")
    tag = pre + case
    a = BSTensor.from_record(rec, tag + ".A")
    b = BSTensor.from_record(rec, tag + ".B")
    ref = BSTensor.from_record(rec, tag + ".C")
    a0, b0, n, sa, sb = _params(rec, tag)
    for mode in _modes(a):
        plan = ContiguousContractionPlan(a, b, a0, b0, n, sa, sb)
        c = plan.execute(DTensor.from_host(a), DTensor.from_host(b), mode=mode)
        plan.device_status()
        c = c.to_host()
        assert same_topology(c, ref), (tag, mode)
        assert rel_frob(c.data, ref.data) <= TOL, (tag, mode)


def test_sides_are_hints(gpu, golden):
    rec = golden("ctrct_contig")
    a = BSTensor.from_record(rec, "f_mid.A")
    b = BSTensor.from_record(rec, "f_mid.B")
    da, db = DTensor.from_host(a), DTensor.from_host(b)
    outs = [ContractContiguousAxes(da, db, 1, 1, 2, sa, sb).to_host()
            for sa in ("head", "tail") for sb in ("head", "tail")]
    for o in outs[1:]:
        assert same_topology(o, outs[0]) and np.array_equal(o.data, outs[0].data)


@pytest.mark.parametrize("pre", ["u_", "f_"])
@pytest.mark.parametrize("case", ACCUM)
def test_accumulate_vs_reference(gpu, golden, pre, case):
    rec = golden("ctrct_contig")
    tag = pre + case
    a = BSTensor.from_record(rec, tag + ".A")
    b = BSTensor.from_record(rec, tag + ".B")
    ref = BSTensor.from_record(rec, tag + ".C")
    c0 = BSTensor.from_record(rec, tag + ".C0") if tag + ".C0.dirs" in rec else None
    a0, b0, n, _, _ = _params(rec, tag)
    al, be = _scalars(rec, tag, a)
    for mode in _modes(a):
        dc = DTensor.from_host(c0) if c0 is not None else None
        out = ContractTailHeadContiguousAccumulate(DTensor.from_host(a), DTensor.from_host(b), a0, b0, n, al, be,
                                                   dc, mode=mode)
        got = out.to_host()
        assert same_topology(got, ref), (tag, mode)
        assert rel_frob(got.data, ref.data) <= TOL, (tag, mode)
        if case in ("acc_same", "acc_superset"):
            assert out is dc   # updated in place: the topology did not grow


@pytest.mark.parametrize("pre", ["u_", "f_"])
def test_try_accumulate_vs_reference(gpu, golden, pre):
    rec = golden("ctrct_contig")
    for case in ("try_fail", "try_ok"):
        tag = pre + case
        a = BSTensor.from_record(rec, tag + ".A")
        b = BSTensor.from_record(rec, tag + ".B")
        ref = BSTensor.from_record(rec, tag + ".C")
        c0 = BSTensor.from_record(rec, tag + ".C0")
        a0, b0, n, _, _ = _params(rec, tag)
        al, be = _scalars(rec, tag, a)
        dc = DTensor.from_host(c0)
        ok, out = TryContractTailHeadContiguousAccumulate(DTensor.from_host(a), DTensor.from_host(b), a0, b0, n,
                                                          al, be, dc)
        assert ok == bool(int(rec[tag + ".ok"][0]))
        got = out.to_host()
        assert same_topology(got, ref)
        if ok:
            assert rel_frob(got.data, ref.data) <= TOL
        else:
            assert np.array_equal(got.data, c0.data)   # untouched


def test_accumulate_errors(gpu, golden):
    rec = golden("ctrct_contig")
    a = BSTensor.from_record(rec, "u_acc_default.A")
    b = BSTensor.from_record(rec, "u_acc_default.B")
    da, db = DTensor.from_host(a), DTensor.from_host(b)
    # a default output needs beta == 0 (the reference throws std::invalid_argument)
    with pytest.raises(capi.QltgError):
        ContractTailHeadContiguousAccumulate(da, db, 2, 0, 1, 1.0, 0.5, None)
    # an output whose indexes are not the result's is a layout mismatch (u_mid.C: rank 4)
    wrong = BSTensor.from_record(rec, "u_mid.C")
    with pytest.raises(capi.ContractAccumulateLayoutMismatch):
        AccumulatePlan(a, b, 2, 0, 1, wrong)
    ok, _ = TryContractTailHeadContiguousAccumulate(da, db, 2, 0, 1, 1.0, 1.0, DTensor.from_host(wrong))
    assert not ok


def test_accumulate_chain_vs_oracle(gpu, golden):
    """Three accumulations in a row (beta = 1: a sum of products, as an environment update
    adds terms) against the oracle, in both modes."""
    rec = golden("ctrct_contig")
    a = BSTensor.from_record(rec, "u_acc_same.A")
    b = BSTensor.from_record(rec, "u_acc_same.B")
    c0 = BSTensor.from_record(rec, "u_acc_same.C0")
    for mode in ("fp64", "split"):
        ref = c0
        dc = DTensor.from_host(c0)
        for alpha in (0.5, -1.25, 2.0):
            _, ref = oracle.accumulate(a, b, 2, 0, 1, alpha, 1.0, ref)
            dc = ContractTailHeadContiguousAccumulate(DTensor.from_host(a), DTensor.from_host(b), 2, 0, 1, alpha, 1.0,
                                                      dc, mode=mode)
        got = dc.to_host()
        assert same_topology(got, ref)
        assert rel_frob(got.data, ref.data) <= TOL
