"""qlten::dmrg axis primitives on the GPU, through the C ABI, against the reference's own
outputs (tests/golden/axis_ops.npz) and the oracle (oracle/axis_ops.py).

Bar: topology identical; scalings within 1e-15 relative (one multiply per element), rank-2
applies within 1e-12 relative Frobenius (FP64 and split precision)."""
import numpy as np
import pytest

from oracle import axis_ops
from tensortoolkit_gb300 import capi
from tensortoolkit_gb300.api import (ApplyAxisDiagonal, ApplyAxisDiagonalInPlace, ApplyAxisMonomial,
                                     ApplyAxisSectorScalars, ApplyRank2ToAxisPreserveOrder,
                                     ApplyTwoRank2ToAxesPreserveOrder, AxisMonomialPlan, AxisRank2Plan, DTensor)
from tensortoolkit_gb300.tensor import BSTensor, rel_frob, same_topology

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def rec(golden):
    return golden("axis_ops")


def _t(rec, p):
    return BSTensor.from_record(rec, p)


@pytest.mark.parametrize("axis", [1, 3])
def test_diagonal_vs_reference(gpu, rec, axis):
    psi = _t(rec, "psi")
    vals = rec[f"diag{axis}.values"]
    dp = DTensor.from_host(psi)
    out = ApplyAxisDiagonal(dp, axis, vals, 1.5, 0.0)
    ref = _t(rec, f"diag{axis}.out")
    got = out.to_host()
    assert same_topology(got, ref) and rel_frob(got.data, ref.data) <= 1e-15
    acc = ApplyAxisDiagonal(dp, axis, vals, -2.0, 0.5, out=out)
    ref2 = _t(rec, f"diag{axis}.acc")
    got2 = acc.to_host()
    assert rel_frob(got2.data, ref2.data) <= 1e-15
    # in place: the tensor scaled by D
    ip = ApplyAxisDiagonalInPlace(DTensor.from_host(psi), axis, vals).to_host()
    assert rel_frob(ip.data, axis_ops.axis_diagonal(psi, axis, vals).data) <= 1e-15


def test_sector_scalars_vs_reference(gpu, rec):
    psi = _t(rec, "psi")
    got = ApplyAxisSectorScalars(DTensor.from_host(psi), 0, rec["sect.values"]).to_host()
    ref = _t(rec, "sect.out")
    assert same_topology(got, ref) and rel_frob(got.data, ref.data) <= 1e-15


@pytest.mark.parametrize("axis", [0, 2, 3])
def test_rank2_vs_reference(gpu, rec, axis):
    psi = _t(rec, "psi")
    op = _t(rec, f"r2_{axis}.op")
    ref = _t(rec, f"r2_{axis}.out")
    for mode in ("fp64", "split"):
        plan = AxisRank2Plan(psi, op, axis)
        got = plan.execute(DTensor.from_host(psi), DTensor.from_host(op), mode=mode)
        plan.device_status()
        got = got.to_host()
        assert same_topology(got, ref), (axis, mode)
        assert all(a.same_space(b) for a, b in zip(got.legs, ref.legs))
        assert rel_frob(got.data, ref.data) <= 1e-12, (axis, mode)


def test_two_rank2_vs_reference(gpu, rec):
    psi = _t(rec, "psi")
    op1, op2 = _t(rec, "two.op1"), _t(rec, "two.op2")
    ref = _t(rec, "two.out")
    for mode in ("fp64", "split"):
        got = ApplyTwoRank2ToAxesPreserveOrder(DTensor.from_host(psi), DTensor.from_host(op1), 0,
                                               DTensor.from_host(op2), 3, mode=mode).to_host()
        assert same_topology(got, ref) and rel_frob(got.data, ref.data) <= 1e-12


@pytest.mark.parametrize("tag", ["mono_p", "mono_b"])
def test_monomial_vs_reference(gpu, rec, tag):
    """A raising map on the physical leg (flux +1) and a permuting, accumulating map inside the
    bond sectors (flux 0): out = 1.25 M(psi), then acc = -0.5 M(psi) + 2 out."""
    psi = _t(rec, "psi")
    axis, flux = (int(x) for x in rec[tag + ".params"])
    ent = rec[tag + ".entries"].reshape(-1, 4)
    coefs = rec[tag + ".coefs"]
    leg = psi.legs[axis]
    dp = DTensor.from_host(psi)
    plan = AxisMonomialPlan(psi, axis, leg, [flux], ent, coefs)
    out = plan.execute(dp, 1.25, 0.0)
    ref = _t(rec, tag + ".out")
    got = out.to_host()
    assert same_topology(got, ref) and rel_frob(got.data, ref.data) <= 1e-15
    acc = ApplyAxisMonomial(dp, axis, leg, [flux], ent, coefs, -0.5, 2.0, out=out)
    ref2 = _t(rec, tag + ".acc")
    got2 = acc.to_host()
    assert same_topology(got2, ref2) and rel_frob(got2.data, ref2.data) <= 1e-15


def test_monomial_flux_mismatch_rejected(gpu, rec):
    psi = _t(rec, "psi")
    with pytest.raises(capi.QltgError):
        AxisMonomialPlan(psi, 1, psi.legs[1], [0], [[0, 0, 1, 0]], [1.0])


def test_rank2_large_vs_oracle(gpu):
    """A D=2000 matvec psi, rank-2 operator on the middle leg (rank-2 ops on a bond leg are the
    environment/truncation updates): GPU vs the oracle."""
    from tensortoolkit_gb300 import workloads
    _, psi, _, _, _ = workloads.heisenberg(600, 8, 3.0, 2)
    rng = np.random.default_rng(1)
    leg = psi.legs[3]
    from tensortoolkit_gb300.tensor import Leg
    new = Leg(leg.dir, leg.qns.copy(), np.maximum(1, leg.dims - 1), leg.parity_comp)
    inv = leg.inverse()
    coords = [[s, s] for s in range(leg.nsct)]
    sizes = [int(leg.dims[s] * new.dims[s]) for s in range(leg.nsct)]
    op = BSTensor([inv, new], np.array(coords), np.float64, rng.standard_normal(sum(sizes)))
    ref = axis_ops.axis_rank2(psi, op, 3)
    got = ApplyRank2ToAxisPreserveOrder(DTensor.from_host(psi), DTensor.from_host(op), 3).to_host()
    assert same_topology(got, ref) and rel_frob(got.data, ref.data) <= 1e-12


def test_fermionic_rejected(gpu, golden):
    rec = golden("qlten_io")
    f = BSTensor.from_record(rec, "f_psi")
    vals = np.ones(int(f.legs[0].dims.sum()))
    with pytest.raises(capi.QltgError):
        ApplyAxisDiagonal(DTensor.from_host(f), 0, vals)
