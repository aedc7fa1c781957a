"""The deterministic workload generator reproduces the reference driver's inputs and the
reference-configuration shapes."""
import numpy as np

from tensortoolkit_gb300 import workloads
from tensortoolkit_gb300.tensor import BSTensor, rel_frob, same_topology


def _same(t: BSTensor, ref: BSTensor):
    assert same_topology(t, ref)
    # bit-identical where libm agrees; allow last-ulp differences from another platform's libm
    assert rel_frob(t.data, ref.data) <= 1e-14


def test_inputs_match_reference_driver(golden):
    rec = golden("matvec_u1_small")
    lenv, psi, mpo1, mpo2, renv = workloads.heisenberg(40, 4, 2.0, 1)
    _same(lenv, BSTensor.from_record(rec, "s1.A"))
    _same(psi, BSTensor.from_record(rec, "s1.B"))
    _same(mpo1, BSTensor.from_record(rec, "s2.B"))
    _same(renv, BSTensor.from_record(rec, "s4.B"))
    rec = golden("matvec_f_small")
    lenv, psi, mpo1, mpo2, renv = workloads.hubbard(24, 2, 4)
    _same(psi, BSTensor.from_record(rec, "s1.B", parity_comp=0))
    assert psi.fermionic and psi.is_complex
    rec = golden("cfg1")
    a, b = workloads.config1(0)
    _same(a, BSTensor.from_record(rec, "c.A"))
    _same(b, BSTensor.from_record(rec, "c.B"))


def test_config_shapes():
    # D=2000, 41 sectors: psi has 160 blocks / 744k elements (reference probe numbers)
    lenv, psi, mpo1, mpo2, renv = workloads.heisenberg(2000, 20, 6.0, 1)
    assert psi.nblk == 160 and abs(psi.size - 744_000) < 2_000
    assert int(psi.legs[0].dims.sum()) == 2000
    lenv, psi, *_ = workloads.heisenberg(4000, 30, 9.0, 1)
    assert psi.nblk == 240 and int(psi.legs[0].dims.sum()) == 4000
    assert abs(np.linalg.norm(psi.data) - 1.0) < 1e-12


def test_hermitian_operands_are_symmetric():
    lenv, psi, mpo1, mpo2, renv = workloads.heisenberg(60, 4, 2.0, 1, hermitian=True)
    L = lenv.to_dense()               # (a, w, a')
    assert np.allclose(L[:, 1:4, :], np.transpose(L[:, 1:4, :], (2, 1, 0)))
    assert np.allclose(L[:, 0, :], L[:, 4, :].T)
    W = mpo1.to_dense()               # (wl, s_in, s_out, wr)
    assert np.count_nonzero(W) == 12  # I x4, S+, S-, Sz x4, S+/2, S-/2
    bar = [4, 1, 2, 3, 0]             # channel involution: q=-1 <-> q=+1, q=0 channels fixed
    assert np.allclose(W[bar][:, :, :, bar].transpose(0, 2, 1, 3), W)
