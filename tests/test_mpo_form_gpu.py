"""The matvec's MPO part in both forms: the two MPO contractions, and one contraction with
W12 = W1 . W2 pre-contracted over the middle MPO bond at creation.

Bar: both forms give the oracle's H psi (topology identical, values within 1e-12 relative
Frobenius) in plain FP64 and in split precision, on the U(1) chain and on the fermionic
complex chain (the fermion signs of the pre-contracted W12 must agree with the two-step
chain); the form chosen at creation is one of the two with its timings recorded; the form
cannot change once the matvec has been applied."""
import pytest

from oracle import oracle
from tensortoolkit_gb300 import workloads
from tensortoolkit_gb300.api import DTensor, Matvec
from tensortoolkit_gb300.capi import QltgError
from tensortoolkit_gb300.tensor import rel_frob, same_topology

pytestmark = pytest.mark.gpu

TOL = 1e-12


@pytest.fixture(scope="module", params=["u1", "fermionic"])
def case(request):
    if request.param == "u1":
        tensors = workloads.heisenberg(1200, 12, 4.0, 2)
    else:
        tensors = workloads.hubbard(900, 6, 5)
    ref, _ = oracle.matvec(*tensors)
    return tensors, ref


@pytest.mark.parametrize("mode", ["fp64", "split"])
@pytest.mark.parametrize("fused", [False, True])
def test_mpo_forms_match_oracle(gpu, case, mode, fused):
    (lenv, psi, mpo1, mpo2, renv), ref = case
    dl, dp, d1, d2, dr = (DTensor.from_host(x) for x in (lenv, psi, mpo1, mpo2, renv))
    mv = Matvec(dl, psi, d1, d2, dr, mode=mode)
    form = mv.mpo_form()
    assert form["fusable"]
    assert form["ms_two_steps"] > 0 and form["ms_fused"] > 0
    mv.set_mpo_form(fused)
    assert mv.mpo_form()["fused"] == fused
    out = mv.apply(dp).to_host()
    mv.device_status()
    assert same_topology(out, ref)
    err = rel_frob(out.data, ref.data)
    assert err <= TOL, (mode, fused, err)
    with pytest.raises(QltgError):
        mv.set_mpo_form(not fused)
