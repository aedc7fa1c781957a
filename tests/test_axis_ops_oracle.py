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


def _kept(rec):
    counts, flat = rec["proj.counts"], rec["proj.kept"]
    starts = np.concatenate([[0], np.cumsum(counts)])
    return [list(flat[starts[s]:starts[s + 1]]) for s in range(len(counts))]


def _close(out, ref, tol=1e-14):
    assert same_topology(out, ref) and rel_frob(out.data, ref.data) <= tol


def test_project(rec):
    _close(axis_ops.project_axis(_t(rec, "psi"), 3, _kept(rec)), _t(rec, "proj.out"), 0.0)


def test_rank2_then_scale(rec):
    psi = _t(rec, "psi")
    r = axis_ops.axis_rank2(psi, _t(rec, "r2diag.op"), 0)
    _close(axis_ops.axis_diagonal(r, 3, rec["r2diag.values"]), _t(rec, "r2diag.out"))
    r = axis_ops.axis_rank2(psi, _t(rec, "r2sect.op"), 3)
    _close(axis_ops.axis_sector_scalars(r, 0, rec["r2sect.values"]), _t(rec, "r2sect.out"))


def _boundary(psi, op, axis, scale_axis, values, alpha, beta, out=None):
    r = axis_ops.axis_sector_scalars(axis_ops.axis_rank2(psi, op, axis), scale_axis, values)
    if out is None:
        return axis_ops.linear_combine([alpha], [r])
    return axis_ops.linear_combine([alpha], [r], beta, out, keep_res=True)


def test_boundary_accumulate(rec):
    psi, op, opp = _t(rec, "psi"), _t(rec, "bnd.op"), _t(rec, "bnd.opp")
    v = rec["bnd.values"]
    fused = _boundary(psi, op, 0, 3, v, 1.0, 0.0)
    _close(fused, _t(rec, "bnd.fused"))
    _close(_boundary(psi, op, 0, 3, v, -0.5, 2.0, _t(rec, "bnd.fused")), _t(rec, "bnd.acc"))
    part = _boundary(psi, opp, 0, 3, v, 1.0, 0.0)
    _close(part, _t(rec, "bnd.part"))
    assert part.nblk < fused.nblk
    _close(_boundary(psi, op, 0, 3, v, 1.25, 0.75, _t(rec, "bnd.part")), _t(rec, "bnd.exp"))
    _close(_boundary(psi, _t(rec, "bnd.op3"), 3, 0, rec["bnd.values0"], 1.0, 0.0), _t(rec, "bnd.last"))


def test_rank2_then_monomial(rec):
    psi = _t(rec, "psi")
    r = axis_ops.axis_rank2(psi, _t(rec, "r2mono.op"), 0)
    ent = rec["mono_b.entries"].reshape(-1, 4)
    out = axis_ops.axis_monomial(r, 3, psi.legs[3], ent, rec["mono_b.coefs"])
    _close(out, _t(rec, "r2mono.out"))


def test_two_rank2_then_scale(rec):
    psi = _t(rec, "psi")
    r = axis_ops.axis_two_rank2(psi, _t(rec, "two2.op1"), 0, _t(rec, "two2.op2"), 3)
    _close(axis_ops.axis_diagonal(r, 1, rec["two2.values"]), _t(rec, "two2.diag"))
    _close(axis_ops.axis_sector_scalars(r, 2, rec["two2.scalars"]), _t(rec, "two2.sect"))


def test_move_head_axis_to_tail(rec):
    psi = _t(rec, "psi")
    _close(axis_ops.transpose(psi, [1, 2, 3, 0]), _t(rec, "move.out"), 0.0)


def test_linear_combine(rec):
    X, Y, Z = _t(rec, "lc.X"), _t(rec, "lc.Y"), _t(rec, "lc.Z")
    assert X.nblk < Z.nblk and Y.nblk < Z.nblk
    _close(axis_ops.linear_combine([1.5, -2.0], [X, Y]), _t(rec, "lc.r1"))
    _close(axis_ops.linear_combine([0.5, 0.0, 3.0], [X, Y, X], 2.0, Z), _t(rec, "lc.r2"))
    _close(axis_ops.linear_combine([0.25], [Y], 1.0, X), _t(rec, "lc.r3"))
