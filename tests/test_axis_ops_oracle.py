"""Pin the CPU restatement of the qlten::dmrg axis primitives (oracle/axis_ops.py) to the
reference's own outputs (tests/golden/axis_ops.npz, made by the reference driver)."""
import numpy as np
import pytest

from oracle import axis_ops
from tensortoolkit_gb300.tensor import BSTensor, rel_frob, same_topology


@pytest.fixture(scope="module")
def rec(golden):
    return golden("axis_ops")


def _t(rec, p):
    return BSTensor.from_record(rec, p)


@pytest.mark.parametrize("axis", [1, 3])
def test_diagonal(rec, axis):
    psi = _t(rec, "psi")
    vals = rec[f"diag{axis}.values"]
    out = axis_ops.axis_diagonal(psi, axis, vals, 1.5, 0.0)
    ref = _t(rec, f"diag{axis}.out")
    assert same_topology(out, ref) and rel_frob(out.data, ref.data) <= 1e-15
    acc = axis_ops.axis_diagonal(psi, axis, vals, -2.0, 0.5, out=ref)
    ref2 = _t(rec, f"diag{axis}.acc")
    assert same_topology(acc, ref2) and rel_frob(acc.data, ref2.data) <= 1e-15


def test_sector_scalars(rec):
    psi = _t(rec, "psi")
    out = axis_ops.axis_sector_scalars(psi, 0, rec["sect.values"])
    ref = _t(rec, "sect.out")
    assert same_topology(out, ref) and rel_frob(out.data, ref.data) <= 1e-15


@pytest.mark.parametrize("axis", [0, 2, 3])
def test_rank2(rec, axis):
    psi = _t(rec, "psi")
    out = axis_ops.axis_rank2(psi, _t(rec, f"r2_{axis}.op"), axis)
    ref = _t(rec, f"r2_{axis}.out")
    assert same_topology(out, ref)
    assert all(a.same_space(b) for a, b in zip(out.legs, ref.legs))
    assert rel_frob(out.data, ref.data) <= 1e-13


def test_two_rank2(rec):
    psi = _t(rec, "psi")
    out = axis_ops.axis_two_rank2(psi, _t(rec, "two.op1"), 0, _t(rec, "two.op2"), 3)
    ref = _t(rec, "two.out")
    assert same_topology(out, ref) and rel_frob(out.data, ref.data) <= 1e-13


@pytest.mark.parametrize("tag", ["mono_p", "mono_b"])
def test_monomial(rec, tag):
    psi = _t(rec, "psi")
    axis, _ = (int(x) for x in rec[tag + ".params"])
    ent = rec[tag + ".entries"].reshape(-1, 4)
    ref = _t(rec, tag + ".out")
    out = axis_ops.axis_monomial(psi, axis, psi.legs[axis], ent, rec[tag + ".coefs"], 1.25, 0.0)
    assert same_topology(out, ref) and rel_frob(out.data, ref.data) <= 1e-15
    acc = axis_ops.axis_monomial(psi, axis, psi.legs[axis], ent, rec[tag + ".coefs"], -0.5, 2.0, out=ref)
    ref2 = _t(rec, tag + ".acc")
    assert same_topology(acc, ref2) and rel_frob(acc.data, ref2.data) <= 1e-15
