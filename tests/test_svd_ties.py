"""SVD truncation through degenerate singular values spread over several block-matrices.

The reference keeps the D largest nonzero singular values of all block-matrices together
(tensor_manipulation/ten_decomp/ten_svd.h:281-372): a descending sort by value, then Dmin
kept and one more while the kept weight stays within (1 - eps) of the total and the count
within Dmax. Equal values across block-matrices keep their order of collection, block-matrix
by block-matrix and rank by rank (the reference's std::sort is an insertion sort at these
sizes, hence stable; the oracle uses a stable sort; the device places every value by counts
under the same order). Spectra are exact here (diagonal blocks of powers of two), so a cut
through a multiplet decides which block-matrix keeps the state without rounding noise.

Bar: kept dimension, truncation error and U / S / Vt topology identical to the oracle and to
the expected kept counts; values within 1e-10."""
import numpy as np
import pytest

from oracle import oracle
from tensortoolkit_gb300.tensor import IN, OUT, BSTensor, Leg
from tests.svd_check import check_svd

SPECTRA = [[1.0, 0.5, 0.25], [0.5, 0.25, 0.125], [0.5, 0.5, 0.0625]]

# kept count per block-matrix for each Dmax (eps = 0: only Dmax cuts), in the global order
# 1 | 0.5 (bm0) 0.5 (bm1) 0.5 0.5 (bm2) | 0.25 (bm0) 0.25 (bm1) | 0.125 | 0.0625
EXPECTED = {1: [1, 0, 0], 2: [2, 0, 0], 3: [2, 1, 0], 4: [2, 1, 1], 5: [2, 1, 2], 6: [3, 1, 2],
            7: [3, 2, 2], 8: [3, 3, 2], 9: [3, 3, 3]}


def _tensor():
    nb = len(SPECTRA)
    left = Leg(IN, np.arange(nb).reshape(-1, 1), np.full(nb, 3))
    right = Leg(OUT, np.arange(nb).reshape(-1, 1), np.full(nb, 3))
    coords = np.array([[i, i] for i in range(nb)], np.int64)
    data = np.concatenate([np.diag(v).reshape(-1) for v in SPECTRA])
    return BSTensor([left, right], coords, np.float64, data)


def _kept_counts(s: BSTensor):
    """Kept count per block-matrix (mid sector qn = the block-matrix's charge)."""
    out = [0] * len(SPECTRA)
    for b in range(s.nblk):
        q = int(s.legs[0].qns[s.coords[b, 0], 0])
        out[q] = int(s.block_shapes()[b][0])
    return out


@pytest.mark.parametrize("dmax", sorted(EXPECTED))
def test_oracle_ties(dmax):
    _, s, _, err, D = oracle.svd(_tensor(), 1, [0], 0.0, 1, dmax)
    assert D == dmax
    assert _kept_counts(s) == EXPECTED[dmax]


@pytest.mark.gpu
@pytest.mark.parametrize("dmax", sorted(EXPECTED))
def test_device_truncation_ties(gpu, dmax):
    from tensortoolkit_gb300.api import SVD, DTensor
    t = _tensor()
    ru, rs, rvt, rerr, rD = oracle.svd(t, 1, [0], 0.0, 1, dmax)
    u, s, vt, err, D = SVD(DTensor.from_host(t), 1, [0], 0.0, 1, dmax)
    s_h = s.to_host()
    assert _kept_counts(s_h) == EXPECTED[dmax]
    check_svd(t, u.to_host(), s_h, vt.to_host(), err, D, ru, rs, rvt, rerr, rD, 1)
