"""Gauge-invariant comparison of block SVD results (shared by CPU and GPU tests)."""
import numpy as np

from tensortoolkit_gb300.tensor import BSTensor, rel_frob, same_topology

SV_TOL = 1e-10


def _dense_by_mid(u: BSTensor, mid_axis: int):
    """For each mid-leg sector coordinate: the dense matrix (other legs fused) x kept."""
    out = {}
    other = [l for l in range(u.rank) if l != mid_axis]
    for b in range(u.nblk):
        mc = int(u.coords[b, mid_axis])
        blk = np.moveaxis(u.block(b), mid_axis, -1)
        key = tuple(int(u.coords[b, l]) for l in other)
        out.setdefault(mc, {})[key] = blk.reshape(-1, blk.shape[-1])
    return {mc: np.concatenate([d[k] for k in sorted(d)], axis=0) for mc, d in out.items()}


def check_svd(t, u, s, vt, err, D, ref_u, ref_s, ref_vt, ref_err, ref_D, ldims):
    assert D == ref_D
    assert abs(err - ref_err) <= 1e-12
    for mine, ref in ((u, ref_u), (s, ref_s), (vt, ref_vt)):
        assert same_topology(mine, ref)
    assert np.max(np.abs(s.data - ref_s.data)) <= SV_TOL
    # singular vectors: per mid sector, columns equal up to a phase where values are simple
    um, ur = _dense_by_mid(u, u.rank - 1), _dense_by_mid(ref_u, ref_u.rank - 1)
    vm, vr = _dense_by_mid(vt, 0), _dense_by_mid(ref_vt, 0)
    svals = {}
    for b in range(s.nblk):
        svals[int(s.coords[b, 0])] = np.diag(s.block(b).reshape(s.block_shapes()[b]))
    for mc in um:
        sv = svals[mc]
        ov_u = np.abs(np.einsum("ij,ij->j", um[mc].conj(), ur[mc]))
        ov_v = np.abs(np.einsum("ij,ij->j", vm[mc].conj(), vr[mc]))
        gap = np.full(len(sv), np.inf)
        if len(sv) > 1:
            d = np.abs(np.diff(sv))
            gap[:-1] = np.minimum(gap[:-1], d)
            gap[1:] = np.minimum(gap[1:], d)
        simple = gap > 1e-6 * max(sv.max(), 1e-300)
        assert np.all(np.abs(ov_u[simple] - 1) < 1e-8), (mc, ov_u[simple].min())
        assert np.all(np.abs(ov_v[simple] - 1) < 1e-8), (mc, ov_v[simple].min())
        # U S Vt agrees with the reference's U S Vt block-matrix by block-matrix
        rec_m = (um[mc] * sv) @ vm[mc].T
        rec_r = (ur[mc] * sv) @ vr[mc].T
        assert rel_frob(rec_m, rec_r) <= 1e-11


