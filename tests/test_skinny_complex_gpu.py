"""Complex contractions whose output blocks all take the FP64 skinny kernel (n, k <= 8), one
per kernel variant the plan picks by its widest block (n <= 2, n <= 4, n <= 8), in both
arithmetic modes, against the oracle; and a real case with the same shapes.

Bar: identical topology, values within 1e-12 relative Frobenius of the oracle."""
import itertools

import numpy as np
import pytest

from oracle import oracle
from tensortoolkit_gb300.api import ContractionPlan, DTensor
from tensortoolkit_gb300.tensor import IN, OUT, BSTensor, Leg, rel_frob, same_topology

pytestmark = pytest.mark.gpu


def _rand(legs, rng, cplx):
    sign = [1 if l.dir == OUT else -1 for l in legs]
    coords = [c for c in itertools.product(*[range(l.nsct) for l in legs])
              if sum(s * int(l.qns[ci, 0]) for s, l, ci in zip(sign, legs, c)) == 0]
    t = BSTensor(legs, np.array(coords, np.int64), np.complex128 if cplx else np.float64)
    if cplx:
        t.data = rng.standard_normal(t.size) + 1j * rng.standard_normal(t.size)
    else:
        t.data = rng.standard_normal(t.size)
    return t


@pytest.mark.parametrize("cplx", [True, False])
@pytest.mark.parametrize("ndims", [(1, 2), (3, 4), (5, 8)])
@pytest.mark.parametrize("mode", ["fp64", "split"])
def test_skinny_blocks_vs_oracle(gpu, cplx, ndims, mode):
    rng = np.random.default_rng(11 + ndims[1])
    L = Leg(IN, np.arange(0, 5).reshape(-1, 1), rng.integers(40, 700, size=5))
    p = Leg(OUT, np.arange(0, 5).reshape(-1, 1), rng.integers(1, 9, size=5))
    q = Leg(OUT, np.arange(0, 5).reshape(-1, 1), rng.integers(ndims[0], ndims[1] + 1, size=5))
    a = _rand([L, p], rng, cplx)
    b = _rand([p.inverse(), q], rng, cplx)
    axes = [[1], [0]]
    ref, _ = oracle.contract(a, b, axes)
    plan = ContractionPlan(a, b, axes)
    got = plan.execute(DTensor.from_host(a), DTensor.from_host(b), mode=mode)
    plan.device_status()
    got = got.to_host()
    assert same_topology(got, ref)
    assert rel_frob(got.data, ref.data) <= 1e-12
