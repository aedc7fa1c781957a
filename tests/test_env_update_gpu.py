"""Left-environment growth of a DMRG sweep (L' = L . psi . W . psi^dagger) as the generic
contraction chain on the GPU, FP64 and split precision, against the oracle chain.

The reference has no environment routine of its own: its callers grow environments with
Contract on the matvec's tensors (tests/test_tensor_manipulation/test_ten_ctrct_1sct.cc:253-257
builds the same first two steps). Bar: topology identical, values within 1e-12 relative
Frobenius."""
import numpy as np
import pytest

from oracle import oracle
from tensortoolkit_gb300 import workloads
from tensortoolkit_gb300.api import ContractionPlan, DTensor
from tensortoolkit_gb300.tensor import BSTensor, rel_frob, same_topology

pytestmark = pytest.mark.gpu

# L (V out, M in, V in) . psi (V in, P in, P in, V out) over (L0, psi0); then the MPO over
# (M, the first P); then psi^dagger over (V, both P): a new L (V out, M in, V in)
CHAIN = [[[0], [0]], [[0, 2], [0, 1]], [[0, 3, 1], [0, 1, 2]]]


def _dagger(t: BSTensor) -> BSTensor:
    return BSTensor([leg.inverse() for leg in t.legs], t.coords, t.dtype, np.conj(t.data))


@pytest.mark.parametrize("mode", ["fp64", "split"])
def test_left_environment_growth(gpu, mode):
    lenv, psi, mpo1, _, _ = workloads.heisenberg(800, 10, 3.0, 3)
    ops = [psi, mpo1, _dagger(psi)]
    ref = lenv
    for b, ax in zip(ops, CHAIN):
        ref, _ = oracle.contract(ref, b, ax)
    assert ref.rank == 3 and all(a.same_space(b) for a, b in zip(ref.legs, lenv.legs))
    cur, cur_meta = DTensor.from_host(lenv), lenv
    for b, ax in zip(ops, CHAIN):
        plan = ContractionPlan(cur_meta, b, ax)
        cur = plan.execute(cur, DTensor.from_host(b), mode=mode)
        plan.device_status()
        cur_meta = plan.result
    got = cur.to_host()
    assert same_topology(got, ref)
    assert rel_frob(got.data, ref.data) <= 1e-12
