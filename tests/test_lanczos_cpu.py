"""The CPU Lanczos itself: on a symmetric two-site H_eff small enough to
build densely, the Ritz values decrease monotonically to the lowest eigenvalue of the dense
matrix, the Krylov basis stays orthonormal, and the synthetic symmetric workload really is
symmetric."""
import numpy as np

from tensortoolkit_gb300 import workloads
from tests.lanczos_ref import lanczos, oracle_apply, ritz_lowest


def small_heff():
    lenv, psi, mpo1, mpo2, renv = workloads.heisenberg(24, 3, 1.5, 5, hermitian=True)
    ops = (lenv, mpo1, mpo2, renv)
    n = psi.size
    H = np.zeros((n, n))
    for i in range(n):
        e = np.zeros(n)
        e[i] = 1.0
        H[:, i] = oracle_apply(ops, psi, e)
    return ops, psi, H


def test_workload_symmetric_and_lanczos_converges():
    ops, psi, H = small_heff()
    print("dimension", psi.size)
    assert np.abs(H - H.T).max() <= 1e-12 * np.abs(H).max()
    e0 = np.linalg.eigvalsh(H)[0]
    x0 = np.random.default_rng(0).standard_normal(psi.size)
    a, b, V = lanczos(lambda x: oracle_apply(ops, psi, x), x0, min(60, psi.size - 1))
    r = ritz_lowest(a, b)
    assert np.all(np.diff(r) <= 1e-10 * abs(e0))          # Ritz values decrease
    assert abs(r[-1] - e0) <= 1e-8 * abs(e0)
    G = V[:-1] @ V[:-1].T
    assert np.abs(G - np.eye(len(G))).max() <= 1e-12


def test_complex_workload_hermitian_and_lanczos_converges():
    """The complex128 U(1) workload's effective Hamiltonian is complex-Hermitian (with a
    non-trivial imaginary part), and the complex CPU Lanczos reaches its lowest eigenvalue."""
    lenv, psi, mpo1, mpo2, renv = workloads.heisenberg_complex_hermitian(24, 3, 1.5, 5)
    ops = (lenv, mpo1, mpo2, renv)
    n = psi.size
    H = np.zeros((n, n), np.complex128)
    for i in range(n):
        e = np.zeros(n, np.complex128)
        e[i] = 1.0
        H[:, i] = oracle_apply(ops, psi, e)
    assert np.abs(H - H.conj().T).max() <= 1e-12 * np.abs(H).max()
    assert np.abs(H.imag).max() >= 0.1 * np.abs(H).max()
    e0 = np.linalg.eigvalsh(H)[0]
    r = np.random.default_rng(0)
    x0 = r.standard_normal(n) + 1j * r.standard_normal(n)
    a, b, V = lanczos(lambda x: oracle_apply(ops, psi, x), x0, min(60, n - 1))
    rz = ritz_lowest(a, b)
    assert np.all(np.diff(rz) <= 1e-10 * abs(e0))
    assert abs(rz[-1] - e0) <= 1e-8 * abs(e0)
    G = V[:-1].conj() @ V[:-1].T
    assert np.abs(G - np.eye(len(G))).max() <= 1e-12
