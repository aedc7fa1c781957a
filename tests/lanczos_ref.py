"""Lanczos with full reorthogonalisation on the CPU oracle's matvec: the reference computation
for the device Lanczos (same recurrence: two passes of classical Gram-Schmidt per step,
alpha_j = Re <v_j, H v_j> including both corrections, beta_{j+1} = ||w||). Real and complex
vectors (<x, y> = sum conj(x) y, the reference's complex Dot, framework/hp_numeric/
blas_level1.h)."""
import numpy as np

from oracle import oracle


def oracle_apply(ops, psi, x):
    """H x for a vector x in psi's layout (oracle matvec); complex psi takes and returns
    complex128 vectors."""
    lenv, mpo1, mpo2, renv = ops
    p = psi.__class__(psi.legs, psi.coords, psi.dtype, np.ascontiguousarray(x), offsets=psi.offsets)
    out, _ = oracle.matvec(lenv, p, mpo1, mpo2, renv)
    y = out.raw_f64().copy()
    return y.view(np.complex128) if psi.is_complex else y


def lanczos(apply, x0, n):
    b0 = np.linalg.norm(x0)
    V = [x0 / b0]
    alpha, beta = [], [b0]
    for j in range(n):
        w = apply(V[j])
        a = 0.0
        for _ in range(2):
            M = np.asarray(V)
            c = M.conj() @ w
            w = w - M.T @ c
            a += c[j].real
        alpha.append(a)
        b = np.linalg.norm(w)
        beta.append(b)
        V.append(w / b if b > 0 else np.zeros_like(w))
    return np.asarray(alpha), np.asarray(beta), np.asarray(V)


def ritz_lowest(alpha, beta):
    out = []
    for k in range(1, len(alpha) + 1):
        T = np.diag(alpha[:k]) + np.diag(beta[1:k], 1) + np.diag(beta[1:k], -1)
        out.append(np.linalg.eigvalsh(T)[0])
    return np.asarray(out)
