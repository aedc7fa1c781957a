"""Device Lanczos against the CPU Lanczos on a symmetric two-site H_eff.

Bar: alpha, beta and the lowest Ritz values of 20 FP64 steps agree with the CPU Lanczos (same
recurrence on the oracle's matvec) to 1e-10 relative; the device Krylov basis is orthonormal
to 1e-12; two runs are bit-identical; the split-precision matvec's Ritz values stay within
1e-10 relative of the FP64 ones (the energy drift the precision study reports)."""
import numpy as np
import pytest
import torch

from tensortoolkit_gb300 import workloads
from tensortoolkit_gb300.api import DTensor, Lanczos, Matvec
from tensortoolkit_gb300.capi import QltgError
from tests.lanczos_ref import lanczos, oracle_apply, ritz_lowest

pytestmark = pytest.mark.gpu

NSTEP = 20


@pytest.fixture(scope="module")
def case():
    lenv, psi, mpo1, mpo2, renv = workloads.heisenberg(200, 10, 3.0, 7, hermitian=True)
    x0 = np.random.default_rng(11).standard_normal(psi.size)
    return (lenv, psi, mpo1, mpo2, renv), x0


def run_device(tensors, x0, mode, n=NSTEP):
    lenv, psi, mpo1, mpo2, renv = tensors
    dl, d1, d2, dr = (DTensor.from_host(x) for x in (lenv, mpo1, mpo2, renv))
    mv = Matvec(dl, psi, d1, d2, dr, mode=mode)
    p0 = DTensor.empty(psi)
    p0.buf[: psi.size].copy_(torch.from_numpy(x0))
    lz = Lanczos(mv, max_iter=n)
    lz.start(p0)
    lz.step(n)
    a, b = lz.coeffs()
    mv.device_status()
    return mv, lz, a, b


def test_lanczos_matches_cpu_lanczos(gpu, case):
    tensors, x0 = case
    lenv, psi, mpo1, mpo2, renv = tensors
    _, _, a, b = run_device(tensors, x0, "fp64")
    ra, rb, _ = lanczos(lambda x: oracle_apply((lenv, mpo1, mpo2, renv), psi, x), x0, NSTEP)
    scale = np.abs(ra).max()
    assert np.abs(a - ra).max() <= 1e-10 * scale
    assert np.abs(b - rb).max() <= 1e-10 * scale
    e, re = ritz_lowest(a, b), ritz_lowest(ra, rb)
    assert np.abs(e - re).max() <= 1e-10 * abs(re[-1])
    assert np.all(np.diff(e) <= 1e-12 * abs(e[-1]))      # Ritz values decrease


def test_krylov_basis_orthonormal(gpu, case):
    tensors, x0 = case
    _, lz, _, _ = run_device(tensors, x0, "fp64")
    V = torch.stack([lz.vector(i) for i in range(NSTEP + 1)])
    G = (V @ V.T).cpu().numpy()
    assert np.abs(G - np.eye(NSTEP + 1)).max() <= 1e-12


def test_lanczos_deterministic(gpu, case):
    tensors, x0 = case
    _, _, a1, b1 = run_device(tensors, x0, "fp64")
    _, _, a2, b2 = run_device(tensors, x0, "fp64")
    assert np.array_equal(a1, a2) and np.array_equal(b1, b2)


def test_split_precision_energy_drift(gpu, case):
    tensors, x0 = case
    _, _, a, b = run_device(tensors, x0, "fp64")
    _, _, sa, sb = run_device(tensors, x0, "split")
    e, es = ritz_lowest(a, b), ritz_lowest(sa, sb)
    drift = np.abs(es - e) / np.abs(e)
    assert drift.max() <= 1e-10, drift


def test_step_limit(gpu, case):
    tensors, x0 = case
    _, lz, _, _ = run_device(tensors, x0, "fp64", n=3)
    with pytest.raises(QltgError):
        lz.step()
