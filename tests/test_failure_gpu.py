"""Failure path of the device-side bounded waits (every mbarrier wait of the tensor-core
kernels gives up after a limit and reports QLTG_ERR_TIMEOUT instead of hanging): a warp waits
on an mbarrier nothing arrives on with a 1 ms limit, the host reads the timeout status, and
the same context then runs split-precision contractions correctly."""
import pytest

from oracle import oracle
from tensortoolkit_gb300 import capi, workloads
from tensortoolkit_gb300.api import ContractionPlan, DTensor, selftest_bounded_wait
from tensortoolkit_gb300.tensor import rel_frob

pytestmark = pytest.mark.gpu


def test_bounded_wait_expires_and_context_survives(gpu):
    for _ in range(2):
        with pytest.raises(capi.QltgError) as e:
            selftest_bounded_wait(1 << 21)        # about 1 ms at 2 GHz
        assert e.value.code == capi.QLTG_ERR_TIMEOUT
    with pytest.raises(capi.QltgError) as e:
        selftest_bounded_wait(0)
    assert e.value.code == capi.QLTG_ERR_INVALID
    a, b = workloads.config1(5)
    ref, _ = oracle.contract(a, b, [[2], [0]])
    plan = ContractionPlan(a, b, [[2], [0]])
    c = plan.execute(DTensor.from_host(a), DTensor.from_host(b), mode="split")
    plan.device_status()
    assert rel_frob(c.to_host().data, ref.data) <= 1e-12
