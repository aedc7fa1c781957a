"""Device Lanczos on complex128 matvecs.

Two workloads:
* a U(1) chain in complex128 whose effective Hamiltonian is complex-Hermitian (environments
  E(a, w, a') = conj(E(a', wbar, a)), the Heisenberg MPO): alpha, beta and the lowest Ritz
  values of 20 FP64 steps agree with the CPU Lanczos (same recurrence, <x, y> = sum conj(x) y,
  on the oracle's matvec) to 1e-10 relative; the device Krylov basis is orthonormal
  (V^H V = I) to 1e-12; the split-precision matvec's Ritz values stay within 1e-10 relative
  of the FP64 ones;
* the fermionic U(1)xU(1) Hubbard-like chain (random complex operands, so H is not
  Hermitian): the same recurrence as the CPU Lanczos to 1e-10 in both precision modes, which
  exercises the complex Gram-Schmidt with the fermion signs of the matvec."""
import numpy as np
import pytest
import torch

from tensortoolkit_gb300 import workloads
from tensortoolkit_gb300.api import DTensor, Lanczos, Matvec
from tests.lanczos_ref import lanczos, oracle_apply, ritz_lowest

pytestmark = pytest.mark.gpu

NSTEP = 20


def _x0(n, seed):
    r = np.random.default_rng(seed)
    return r.standard_normal(n) + 1j * r.standard_normal(n)


@pytest.fixture(scope="module")
def herm():
    tensors = workloads.heisenberg_complex_hermitian(200, 10, 3.0, 7)
    return tensors, _x0(tensors[1].size, 11)


@pytest.fixture(scope="module")
def hubbard():
    tensors = workloads.hubbard(400, 4, 9)
    return tensors, _x0(tensors[1].size, 12)


def run_device(tensors, x0, mode, n=NSTEP):
    lenv, psi, mpo1, mpo2, renv = tensors
    dl, d1, d2, dr = (DTensor.from_host(x) for x in (lenv, mpo1, mpo2, renv))
    mv = Matvec(dl, psi, d1, d2, dr, mode=mode)
    p0 = DTensor.empty(psi)
    p0.buf[: 2 * psi.size].copy_(torch.from_numpy(np.ascontiguousarray(x0).view(np.float64)))
    lz = Lanczos(mv, max_iter=n)
    lz.start(p0)
    lz.step(n)
    a, b = lz.coeffs()
    mv.device_status()
    return mv, lz, a, b


def cpu_lanczos(tensors, x0, n=NSTEP):
    lenv, psi, mpo1, mpo2, renv = tensors
    return lanczos(lambda x: oracle_apply((lenv, mpo1, mpo2, renv), psi, x), x0, n)


def test_complex_hermitian_lanczos_matches_cpu(gpu, herm):
    tensors, x0 = herm
    _, _, a, b = run_device(tensors, x0, "fp64")
    ra, rb, _ = cpu_lanczos(tensors, x0)
    scale = np.abs(ra).max()
    assert np.abs(a - ra).max() <= 1e-10 * scale
    assert np.abs(b - rb).max() <= 1e-10 * scale
    e, re = ritz_lowest(a, b), ritz_lowest(ra, rb)
    assert np.abs(e - re).max() <= 1e-10 * abs(re[-1])
    assert np.all(np.diff(e) <= 1e-12 * abs(e[-1]))      # Ritz values decrease


def test_complex_krylov_basis_orthonormal(gpu, herm):
    tensors, x0 = herm
    _, lz, _, _ = run_device(tensors, x0, "fp64")
    V = torch.stack([lz.vector(i) for i in range(NSTEP + 1)])
    assert V.dtype == torch.complex128
    G = (V.conj() @ V.T).cpu().numpy()
    assert np.abs(G - np.eye(NSTEP + 1)).max() <= 1e-12


def test_complex_split_precision_energy_drift(gpu, herm):
    tensors, x0 = herm
    _, _, a, b = run_device(tensors, x0, "fp64")
    _, _, sa, sb = run_device(tensors, x0, "split")
    e, es = ritz_lowest(a, b), ritz_lowest(sa, sb)
    drift = np.abs(es - e) / np.abs(e)
    assert drift.max() <= 1e-10, drift


@pytest.mark.parametrize("mode", ["fp64", "split"])
def test_fermionic_complex_lanczos_recurrence(gpu, hubbard, mode):
    tensors, x0 = hubbard
    _, lz, a, b = run_device(tensors, x0, mode)
    ra, rb, _ = cpu_lanczos(tensors, x0)
    scale = max(np.abs(ra).max(), np.abs(rb[1:]).max())
    assert np.abs(a - ra).max() <= 1e-10 * scale, (mode, np.abs(a - ra).max() / scale)
    assert np.abs(b - rb).max() <= 1e-10 * scale, (mode, np.abs(b - rb).max() / scale)
    V = torch.stack([lz.vector(i) for i in range(NSTEP + 1)])
    G = (V.conj() @ V.T).cpu().numpy()
    assert np.abs(G - np.eye(NSTEP + 1)).max() <= 1e-12


def test_complex_lanczos_deterministic(gpu, herm):
    tensors, x0 = herm
    _, _, a1, b1 = run_device(tensors, x0, "split")
    _, _, a2, b2 = run_device(tensors, x0, "split")
    assert np.array_equal(a1, a2) and np.array_equal(b1, b2)
