"""Parity of the CUDA contraction path with the reference (golden fixtures) and with the
CPU restatement (full-size cases), through the C ABI.

Bar: block sets, shapes, task lists and fermion signs bit-exact; FP64 values within
1e-12 relative Frobenius error of the reference / oracle."""
import numpy as np
import pytest

from oracle import oracle
from tensortoolkit_gb300 import workloads
from tensortoolkit_gb300.api import Contract, ContractionPlan, DTensor, Matvec, Transpose
from tensortoolkit_gb300.tensor import BSTensor, rel_frob, same_topology

pytestmark = pytest.mark.gpu

TOL = 1e-12   # relative Frobenius, FP64

CTRCT_CASES = [
    ("cfg1", ["c"]),
    ("matvec_u1_small", ["s1", "s2", "s3", "s4"]),
    ("matvec_f_small", ["s1", "s2", "s3", "s4"]),
    ("ctrct_misc_u1", ["u_scalar", "u_perm", "u_mid", "f_scalar", "f_in", "f_rev", "f_env", "f_mpo"]),
]


def _axes(rec, tag):
    ax = rec[tag + ".axes"]
    n = len(ax) // 2
    return [list(ax[:n]), list(ax[n:])]


@pytest.mark.parametrize("case,tags", CTRCT_CASES)
def test_contract_golden(gpu, golden, case, tags):
    rec = golden(case)
    for tag in tags:
        a = BSTensor.from_record(rec, tag + ".A")
        b = BSTensor.from_record(rec, tag + ".B")
        ref = BSTensor.from_record(rec, tag + ".C")
        plan = ContractionPlan(a, b, _axes(rec, tag))
        assert np.array_equal(plan.tasks(), rec[tag + ".tasks"].reshape(-1, 8)), f"{case}/{tag}: tasks"
        c = plan.execute(DTensor.from_host(a), DTensor.from_host(b)).to_host()
        if ref.rank:
            assert same_topology(c, ref), f"{case}/{tag}: topology"
        assert c.size == ref.size
        assert rel_frob(c.data, ref.data) <= TOL, f"{case}/{tag}: {rel_frob(c.data, ref.data)}"


def _check_vs_oracle(a, b, axes):
    ref, ref_tasks = oracle.contract(a, b, axes)
    plan = ContractionPlan(a, b, axes)
    assert np.array_equal(plan.tasks(), ref_tasks)
    c = plan.execute(DTensor.from_host(a), DTensor.from_host(b)).to_host()
    assert same_topology(c, ref)
    err = rel_frob(c.data, ref.data)
    assert err <= TOL, err
    return c


@pytest.mark.parametrize("D,qmax,sigma", [(2000, 20, 6.0), (4000, 30, 9.0)])
def test_matvec_full_size_vs_oracle(gpu, D, qmax, sigma):
    lenv, psi, mpo1, mpo2, renv = workloads.heisenberg(D, qmax, sigma, 1)
    ref, (t1, t2, t3) = oracle.matvec(lenv, psi, mpo1, mpo2, renv)
    dl, dp, d1, d2, dr = (DTensor.from_host(x) for x in (lenv, psi, mpo1, mpo2, renv))
    mv = Matvec(dl, psi, d1, d2, dr, mode="fp64")
    assert same_topology(mv.result, ref)
    out = mv.apply(dp).to_host()
    assert rel_frob(out.data, ref.data) <= TOL
    # the captured graph replays identically
    out2 = mv.apply(dp).to_host()
    assert np.array_equal(out.data, out2.data)


def test_matvec_steps_vs_oracle(gpu):
    lenv, psi, mpo1, mpo2, renv = workloads.heisenberg(600, 8, 3.0, 2)
    t1 = _check_vs_oracle(lenv, psi, [[0], [0]])
    t2 = _check_vs_oracle(t1, mpo1, [[0, 2], [0, 1]])
    t3 = _check_vs_oracle(t2, mpo2, [[4, 1], [0, 1]])
    _check_vs_oracle(t3, renv, [[4, 1], [1, 0]])


def test_fermionic_complex_vs_oracle(gpu):
    lenv, psi, mpo1, mpo2, renv = workloads.hubbard(1200, 10, 4)
    ref, _ = oracle.matvec(lenv, psi, mpo1, mpo2, renv)
    t1 = _check_vs_oracle(lenv, psi, [[0], [0]])
    t2 = _check_vs_oracle(t1, mpo1, [[0, 2], [0, 1]])
    dl, dp, d1, d2, dr = (DTensor.from_host(x) for x in (lenv, psi, mpo1, mpo2, renv))
    out = Matvec(dl, psi, d1, d2, dr).apply(dp).to_host()
    assert same_topology(out, ref)
    assert rel_frob(out.data, ref.data) <= TOL


def test_fermionic_complex_matvec_d6000_vs_oracle(gpu):
    """The fermionic U(1)xU(1) complex128 matvec at its full size (D=6000, 400 bond sectors)
    in plain FP64 against the oracle: identical topology, values within 1e-12."""
    lenv, psi, mpo1, mpo2, renv = workloads.hubbard(6000, 10, 4)
    ref, _ = oracle.matvec(lenv, psi, mpo1, mpo2, renv)
    dl, dp, d1, d2, dr = (DTensor.from_host(x) for x in (lenv, psi, mpo1, mpo2, renv))
    mv = Matvec(dl, psi, d1, d2, dr, mode="fp64")
    out = mv.apply(dp).to_host()
    mv.device_status()
    assert same_topology(out, ref)
    err = rel_frob(out.data, ref.data)
    print(f"complex D=6000 FP64 vs oracle rel Frobenius {err:.3e}")
    assert err <= TOL


def test_matvec_linearity_full_size(gpu):
    """Size-independent property at the benchmark size: H(x psi1 + y psi2) = x H psi1 + y H psi2."""
    import torch
    lenv, psi, mpo1, mpo2, renv = workloads.heisenberg(4000, 30, 9.0, 1)
    dl, d1, d2, dr = (DTensor.from_host(x) for x in (lenv, mpo1, mpo2, renv))
    mv = Matvec(dl, psi, d1, d2, dr)
    p1 = DTensor.from_host(psi)
    p2 = DTensor.empty(psi)
    p2.buf.copy_(torch.randn_like(p1.buf))
    p3 = DTensor.empty(psi)
    p3.buf.copy_(0.3 * p1.buf - 1.7 * p2.buf)
    h1, h2, h3 = mv.apply(p1).buf.clone(), mv.apply(p2).buf.clone(), mv.apply(p3).buf.clone()
    ref = 0.3 * h1 - 1.7 * h2
    assert float(torch.linalg.norm(h3 - ref) / torch.linalg.norm(ref)) <= 1e-13


def test_no_pairs_gives_empty_result(gpu, golden):
    rec = golden("cfg1")
    a = BSTensor.from_record(rec, "c.A")
    b = BSTensor.from_record(rec, "c.B")
    # keep only A blocks whose contracted sector has no partner in B
    keep = np.isin(a.coords[:, 2], [5])
    bb_keep = ~np.isin(b.coords[:, 0], [5])
    a2 = BSTensor(a.legs, a.coords[keep], a.dtype, np.concatenate([a.block(i).ravel() for i in np.where(keep)[0]]))
    b2 = BSTensor(b.legs, b.coords[bb_keep], b.dtype,
                  np.concatenate([b.block(i).ravel() for i in np.where(bb_keep)[0]]))
    plan = ContractionPlan(a2, b2, [[2], [0]])
    assert plan.result.nblk == 0 and plan.result.size == 0
    assert plan.tasks().shape == (0, 8)


def test_invalid_axes_rejected(gpu, golden):
    from tensortoolkit_gb300.capi import QltgError
    rec = golden("cfg1")
    a = BSTensor.from_record(rec, "c.A")
    b = BSTensor.from_record(rec, "c.B")
    with pytest.raises(QltgError):
        ContractionPlan(a, b, [[0], [0]])     # A.leg0 is not the inverse of B.leg0
    with pytest.raises(QltgError):
        ContractionPlan(a, b, [[2, 2], [0, 0]])


def _reorder_sign(par, order):
    # FermionicInplaceReorder (reference utility/utils_inl.h:52-75), restated for the test
    idx = list(order)
    par = list(par)
    ex = 0
    for i in range(len(idx)):
        cur = i
        while i != idx[cur]:
            nxt = idx[cur]
            between = sum(par[j] for j in range(min(cur, nxt) + 1, max(cur, nxt)))
            ex += between * (par[cur] + par[nxt]) + par[cur] * par[nxt]
            par[cur], par[nxt] = par[nxt], par[cur]
            idx[cur] = cur
            cur = nxt
        idx[cur] = cur
    return -1 if ex & 1 else 1


def test_reorder_sign_known_answers():
    # reference tests/test_utility/test_fermion_parity_exchange.cc:14-35
    assert _reorder_sign([1, 0, 1, 0], [2, 1, 3, 0]) == -1
    assert _reorder_sign([1, 1, 1, 0], [3, 1, 0, 2]) == -1


@pytest.mark.parametrize("perm", [(0, 2, 3, 1), (3, 2, 1, 0), (1, 0, 2, 3), (0, 1, 3, 2)])
def test_transpose_with_fermion_signs(gpu, perm):
    lenv, psi, *_ = workloads.hubbard(300, 4, 9)
    out = Transpose(DTensor.from_host(psi), perm).to_host()
    # expected: dense permutation with the per-block exchange sign
    for b in range(psi.nblk):
        coords = psi.coords[b]
        par = [psi.legs[l].parities()[coords[l]] for l in range(4)]
        sgn = _reorder_sign(par, perm)
        new = coords[list(perm)]
        ob = np.where((out.coords == new).all(axis=1))[0]
        assert len(ob) == 1
        np.testing.assert_array_equal(out.block(int(ob[0])), sgn * np.transpose(psi.block(b), perm))


def test_transpose_large_blocks(gpu):
    lenv, psi, mpo1, mpo2, renv = workloads.heisenberg(4000, 30, 9.0, 1)
    t = DTensor.from_host(lenv)
    out = Transpose(t, (2, 1, 0)).to_host()
    for b in range(0, lenv.nblk, 7):
        c = lenv.coords[b]
        ob = np.where((out.coords == c[[2, 1, 0]]).all(axis=1))[0][0]
        np.testing.assert_array_equal(out.block(int(ob)), np.transpose(lenv.block(b), (2, 1, 0)))


@pytest.mark.parametrize("perm", [(0, 2, 3, 1), (3, 2, 1, 0)])
def test_transpose_plan_matches_transpose(gpu, perm):
    """A reusable plan gives Transpose's result bit for bit, on repeated executions and on a
    second tensor of the same layout (fermionic complex tensor: block signs included)."""
    from tensortoolkit_gb300.api import TransposePlan
    lenv, psi, *_ = workloads.hubbard(300, 4, 9)
    d = DTensor.from_host(psi)
    plan = TransposePlan(psi, perm)
    ref = Transpose(d, perm).to_host()
    for _ in range(2):
        got = plan.execute(d).to_host()
        np.testing.assert_array_equal(got.coords, ref.coords)
        np.testing.assert_array_equal(got.data, ref.data)
    psi2 = BSTensor(psi.legs, psi.coords, psi.dtype, psi.data * 2.0)
    got2 = plan.execute(DTensor.from_host(psi2)).to_host()
    np.testing.assert_array_equal(got2.data, ref.data * 2.0)
