"""Pin the oracle's complex128 block SVD and QR, which the reference's fixtures (all real)
do not cover: on the fermionic fU(1) x U(1) Hubbard psi the untruncated factors must
rebuild the tensor under the reference's own Contract semantics (fermion signs included;
that contraction is pinned to the reference's fixtures), U and Q must have orthonormal
columns per block-matrix, and the singular values must equal numpy's (LAPACK) on each
densified block-matrix. The same reconstruction check is first run on the reference's own
fixtures (its fermionic QR, its untruncated SVD), so the property itself is pinned.

Bar: reconstruction within 1e-12 relative Frobenius; singular values within 1e-12 of the
largest; Q^H Q and U^H U within 1e-12 of the identity."""
import numpy as np
import pytest

from oracle import oracle
from tensortoolkit_gb300 import workloads
from tensortoolkit_gb300.tensor import BSTensor, rel_frob


def _by_coords(t: BSTensor):
    return {tuple(int(x) for x in t.coords[b]): t.block(b) for b in range(t.nblk)}


def _rebuilt_matches(t: BSTensor, r: BSTensor, tol: float):
    """r equals t blockwise: same nonzero blocks, values within tol (relative Frobenius)."""
    bt, br = _by_coords(t), _by_coords(r)
    keys = set(bt) | set(br)
    num = den = 0.0
    for k in keys:
        x = bt.get(k)
        y = br.get(k)
        if x is None:
            x = np.zeros_like(y)
        if y is None:
            y = np.zeros_like(x)
        num += float(np.sum(np.abs(x - y) ** 2))
        den += float(np.sum(np.abs(x) ** 2))
    return np.sqrt(num / max(den, 1e-300)) <= tol


def _columns_by_mid(u: BSTensor, mid_axis: int):
    """Per mid-leg sector: the dense matrix of the other legs (fused) x kept columns."""
    out = {}
    other = [l for l in range(u.rank) if l != mid_axis]
    for b in range(u.nblk):
        mc = int(u.coords[b, mid_axis])
        blk = np.moveaxis(u.block(b), mid_axis, -1)
        key = tuple(int(u.coords[b, l]) for l in other)
        out.setdefault(mc, {})[key] = blk.reshape(-1, blk.shape[-1])
    return {mc: np.concatenate([d[k] for k in sorted(d)], axis=0) for mc, d in out.items()}


def _check_svd_rebuild(t, ldims):
    u, s, vt, err, D = oracle.svd(t, ldims, [0] * t.ncomp, 0.0, 1, 10 ** 9)
    assert err == 0.0
    sc = s if not u.is_complex else BSTensor(s.legs, s.coords, np.complex128, s.data.astype(np.complex128))
    us, _ = oracle.contract(u, sc, [[ldims], [0]])
    r, _ = oracle.contract(us, vt, [[ldims], [0]])
    assert _rebuilt_matches(t, r, 1e-12)
    for mc, m in _columns_by_mid(u, u.rank - 1).items():
        assert np.abs(m.conj().T @ m - np.eye(m.shape[1])).max() <= 1e-12, mc
    return u, s, vt


def _check_qr_rebuild(t, ldims):
    q, r = oracle.qr(t, ldims, [0] * t.ncomp)
    back, _ = oracle.contract(q, r, [[ldims], [0]])
    assert _rebuilt_matches(t, back, 1e-12)
    for mc, m in _columns_by_mid(q, q.rank - 1).items():
        assert np.abs(m.conj().T @ m - np.eye(m.shape[1])).max() <= 1e-12, mc


def test_reconstruction_property_on_reference_fixtures(golden):
    """The reference's own outputs rebuild their input under Contract: its fermionic QR, and
    its untruncated SVD (svd_u1_full keeps every nonzero singular value: error 0)."""
    for case, names in (("qr_f", ("Q", "R")), ("svd_u1_full", ("U", "S", "Vt"))):
        rec = golden(case)
        t = BSTensor.from_record(rec, "T")
        ldims = int(rec["ldims"][0])
        f = [BSTensor.from_record(rec, n) for n in names]
        x, _ = oracle.contract(f[0], f[1], [[ldims], [0]])
        if len(f) == 3:
            assert float(rec["err"][0]) == 0.0
            x, _ = oracle.contract(x, f[2], [[ldims], [0]])
        assert _rebuilt_matches(t, x, 1e-12), case


@pytest.mark.parametrize("D", [400, 1200])
def test_complex_fermionic_svd_rebuilds_and_matches_lapack(D):
    _, psi, *_ = workloads.hubbard(D)
    assert psi.is_complex and psi.fermionic
    u, s, vt = _check_svd_rebuild(psi, 2)
    # singular values of each block-matrix = numpy's on the densified block-matrix U S Vt
    um, vm = _columns_by_mid(u, u.rank - 1), _columns_by_mid(vt, 0)
    for b in range(s.nblk):
        mc = int(s.coords[b, 0])
        sv = np.diag(s.block(b).reshape(s.block_shapes()[b]))
        dense = (um[mc] * sv) @ vm[mc].T
        ref = np.linalg.svd(dense, compute_uv=False)[: len(sv)]
        assert np.abs(np.sort(sv)[::-1] - ref).max() <= 1e-12 * max(ref.max(), 1.0)


@pytest.mark.parametrize("D", [400, 1200])
def test_complex_fermionic_qr_rebuilds(D):
    _, psi, *_ = workloads.hubbard(D)
    _check_qr_rebuild(psi, 2)
