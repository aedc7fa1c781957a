"""qlten::dmrg axis primitives on the GPU, through the C ABI, against the reference's own
outputs (tests/golden/axis_ops.npz) and the oracle (oracle/axis_ops.py).

Bar: topology identical; scalings within 1e-15 relative (one multiply per element), rank-2
applies within 1e-12 relative Frobenius (FP64 and split precision)."""
import numpy as np
import pytest

from oracle import axis_ops
from tensortoolkit_gb300 import capi
from tensortoolkit_gb300 import api
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


def _d(rec, p):
    return DTensor.from_host(_t(rec, p))


def _close(got: DTensor, ref: BSTensor, tol=1e-12):
    g = got.to_host()
    assert same_topology(g, ref) and all(a.same_space(b) for a, b in zip(g.legs, ref.legs))
    assert rel_frob(g.data, ref.data) <= tol


def test_project_vs_reference(gpu, rec):
    counts, flat = rec["proj.counts"], rec["proj.kept"]
    starts = np.concatenate([[0], np.cumsum(counts)])
    kept = [list(flat[starts[s]:starts[s + 1]]) for s in range(len(counts))]
    _close(api.ProjectAxis(_d(rec, "psi"), 3, kept), _t(rec, "proj.out"), 0.0)
    with pytest.raises(capi.QltgError):   # an offset kept twice
        api.ProjectAxis(_d(rec, "psi"), 3, [[0, 0]] + kept[1:])


@pytest.mark.parametrize("mode", ["fp64", "split"])
def test_rank2_then_scale_vs_reference(gpu, rec, mode):
    psi = _d(rec, "psi")
    _close(api.ApplyRank2ThenAxisDiagonalPreserveOrder(psi, _d(rec, "r2diag.op"), 0, 3, rec["r2diag.values"], mode),
           _t(rec, "r2diag.out"))
    _close(api.ApplyRank2ThenAxisSectorScalarsPreserveOrder(psi, _d(rec, "r2sect.op"), 3, 0, rec["r2sect.values"],
                                                            mode), _t(rec, "r2sect.out"))


def test_boundary_accumulate_vs_reference(gpu, rec):
    psi, op, opp = _d(rec, "psi"), _d(rec, "bnd.op"), _d(rec, "bnd.opp")
    v = rec["bnd.values"]
    f = api.ApplyBoundaryRank2ThenAxisSectorScalarsFusedPreserveOrder
    acc = api.ApplyBoundaryRank2ThenAxisSectorScalarsAccumulatePreserveOrder
    fused = f(psi, op, 0, 3, v)
    _close(fused, _t(rec, "bnd.fused"))
    upd = acc(psi, op, 0, 3, v, -0.5, 2.0, fused)
    assert upd is fused   # same topology: updated in place
    _close(upd, _t(rec, "bnd.acc"))
    part = f(psi, opp, 0, 3, v)
    _close(part, _t(rec, "bnd.part"))
    _close(acc(psi, op, 0, 3, v, 1.25, 0.75, part), _t(rec, "bnd.exp"))
    _close(f(psi, _d(rec, "bnd.op3"), 3, 0, rec["bnd.values0"]), _t(rec, "bnd.last"))
    with pytest.raises(ValueError):   # a middle axis is not a boundary
        f(psi, _d(rec, "r2_2.op"), 2, 0, rec["bnd.values0"])


def test_rank2_then_monomial_vs_reference(gpu, rec):
    psi = _t(rec, "psi")
    out = api.ApplyRank2ThenAxisMonomialFusedPreserveOrder(DTensor.from_host(psi), _d(rec, "r2mono.op"), 0, 3,
                                                           psi.legs[3], [0], rec["mono_b.entries"].reshape(-1, 4),
                                                           rec["mono_b.coefs"])
    _close(out, _t(rec, "r2mono.out"))


def test_two_rank2_then_scale_vs_reference(gpu, rec):
    psi, op1, op2 = _d(rec, "psi"), _d(rec, "two2.op1"), _d(rec, "two2.op2")
    _close(api.ApplyTwoRank2ThenAxisDiagonalPreserveOrder(psi, op1, 0, op2, 3, 1, rec["two2.values"]),
           _t(rec, "two2.diag"))
    _close(api.ApplyTwoRank2ThenAxisSectorScalarsPreserveOrder(psi, op1, 0, op2, 3, 2, rec["two2.scalars"]),
           _t(rec, "two2.sect"))


def test_move_head_axis_to_tail_vs_reference(gpu, rec):
    _close(api.MoveHeadAxisToTail(_d(rec, "psi")), _t(rec, "move.out"), 0.0)


def test_scale_forms(gpu, rec):
    psi = _t(rec, "psi")
    d = DTensor.from_host(psi)
    out = api.ScaleAxisSectorsInPlace(d, 0, rec["sect.values"])
    assert out is d
    _close(out, _t(rec, "sect.out"), 1e-15)
    vals = rec["diag3.values"]
    a = api.ApplyAxisDiagonalPreserveOrder(DTensor.from_host(psi), 3, vals)
    b = api.ApplyAxisDiagonalPreserveOrder(DTensor.from_host(psi), 3, vals, in_place=True)
    ref = axis_ops.axis_diagonal(psi, 3, vals)
    _close(a, ref, 1e-15)
    _close(b, ref, 1e-15)


def test_linear_combine_vs_reference(gpu, rec):
    X, Y, Z = _d(rec, "lc.X"), _d(rec, "lc.Y"), _d(rec, "lc.Z")
    _close(api.LinearCombine([1.5, -2.0], [X, Y]), _t(rec, "lc.r1"), 1e-15)
    z = _d(rec, "lc.Z")
    r2 = api.LinearCombine([0.5, 0.0, 3.0], [X, Y, X], 2.0, z)
    assert r2 is z   # union of X and Z is Z's topology: written in place
    _close(r2, _t(rec, "lc.r2"), 1e-15)
    _close(api.AddScaledAssign(_d(rec, "lc.X"), 0.25, Y), _t(rec, "lc.r3"), 1e-15)
    with pytest.raises(capi.QltgError):   # beta != 0 without a result tensor
        api.LinearCombine([1.0], [X], 1.0, None)
    with pytest.raises(capi.ContractAccumulateLayoutMismatch):   # other indexes
        api.LinearCombine([1.0, 1.0], [X, _d(rec, "psi")])


def test_linear_combine_complex_vs_oracle(gpu):
    """Complex tensors with different block sets against the numpy restatement."""
    from tensortoolkit_gb300 import workloads
    _, psi, _, _, _ = workloads.hubbard(40)
    rng = np.random.default_rng(4)
    ts = []
    for k in range(3):
        keep = np.sort(rng.choice(psi.nblk, size=max(1, psi.nblk // 2), replace=False))
        t = BSTensor(psi.legs, psi.coords[keep], np.complex128)
        t.data = rng.standard_normal(t.size) + 1j * rng.standard_normal(t.size)
        ts.append(t)
    coefs = [1.0 - 0.5j, 0.0, 2.0 + 1.0j]
    res = ts[1]
    ref = axis_ops.linear_combine(coefs, ts, 0.5 + 0.25j, res)
    got = api.LinearCombine(coefs, [DTensor.from_host(t) for t in ts], 0.5 + 0.25j, DTensor.from_host(res))
    _close(got, ref, 1e-15)


def test_linear_combine_limits_and_aliasing(gpu, rec):
    X = _d(rec, "lc.X")
    ref = _t(rec, "lc.X")
    # 64 tensors (the most one plan takes), then 65
    got = api.LinearCombine([1.0] * 64, [X] * 64).to_host()
    assert same_topology(got, ref) and rel_frob(got.data, 64.0 * ref.data) <= 1e-15
    with pytest.raises(capi.QltgError):
        api.LinearCombine([1.0] * 65, [X] * 65)
    # y += 0.5 y in place
    y = _d(rec, "lc.X")
    out = api.AddScaledAssign(y, 0.5, y)
    assert out is y and rel_frob(y.to_host().data, 1.5 * ref.data) <= 1e-15
    with pytest.raises(ValueError):   # complex coefficient for a real tensor
        api.LinearCombine([1.0 + 1.0j], [X])


def test_project_errors(gpu, rec):
    psi = _d(rec, "psi")
    nsct = _t(rec, "psi").legs[3].nsct
    with pytest.raises(capi.QltgError):   # nothing kept
        api.ProjectAxis(psi, 3, [[] for _ in range(nsct)])
    with pytest.raises(capi.QltgError):   # offset outside its sector
        api.ProjectAxis(psi, 3, [[5]] + [[] for _ in range(nsct - 1)])
