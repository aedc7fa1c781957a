"""Split-precision contraction (FP64 emulated with BF16 slices on the tcgen05 tensor cores)
against the reference (golden fixtures) and the FP64 oracle.

Bar: block topology and task lists identical to the FP64 path; relative Frobenius error of
the full result <= 1e-12 against the FP64 reference / oracle, per-block errors reported and
bounded; no expired device wait."""
import numpy as np
import pytest

from oracle import oracle
from tensortoolkit_gb300 import workloads
from tensortoolkit_gb300.api import ContractionPlan, DTensor, Matvec
from tensortoolkit_gb300.tensor import BSTensor, rel_frob, same_topology

pytestmark = pytest.mark.gpu

TOL = 1e-12          # whole result, relative Frobenius
TOL_BLOCK = 1e-11    # any single block, relative Frobenius (small blocks see less averaging)


def block_errors(c: BSTensor, ref: BSTensor) -> np.ndarray:
    errs = []
    for b in range(ref.nblk):
        x, y = c.block(b), ref.block(b)
        n = np.linalg.norm(y)
        errs.append(np.linalg.norm(x - y) / n if n > 0 else np.linalg.norm(x))
    return np.asarray(errs)


CASES = [("cfg1", ["c"]), ("matvec_u1_small", ["s1", "s2", "s3", "s4"]),
         ("ctrct_misc_u1", ["u_scalar", "u_perm", "u_mid"]),
         # fermionic complex128: the real 2k x 2n embedding of complex B
         ("matvec_f_small", ["s1", "s2", "s3", "s4"]),
         ("ctrct_misc_u1", ["f_env", "f_in", "f_mpo", "f_rev", "f_scalar"])]


@pytest.mark.parametrize("case,tags", CASES)
def test_split_golden(gpu, golden, case, tags):
    rec = golden(case)
    for tag in tags:
        a = BSTensor.from_record(rec, tag + ".A")
        b = BSTensor.from_record(rec, tag + ".B")
        ref = BSTensor.from_record(rec, tag + ".C")
        ax = rec[tag + ".axes"]
        n = len(ax) // 2
        plan = ContractionPlan(a, b, [list(ax[:n]), list(ax[n:])])
        c = plan.execute(DTensor.from_host(a), DTensor.from_host(b), mode="split")
        plan.device_status()
        c = c.to_host()
        if ref.rank:
            assert same_topology(c, ref)
        err = rel_frob(c.data, ref.data)
        assert err <= TOL, (case, tag, err)


@pytest.mark.parametrize("D,qmax,sigma", [(2000, 20, 6.0), (4000, 30, 9.0)])
def test_split_matvec_vs_fp64_oracle(gpu, D, qmax, sigma):
    lenv, psi, mpo1, mpo2, renv = workloads.heisenberg(D, qmax, sigma, 1)
    ref, _ = oracle.matvec(lenv, psi, mpo1, mpo2, renv)
    dl, dp, d1, d2, dr = (DTensor.from_host(x) for x in (lenv, psi, mpo1, mpo2, renv))
    mv = Matvec(dl, psi, d1, d2, dr, mode="split")
    out = mv.apply(dp)
    mv.device_status()
    out = out.to_host()
    assert same_topology(out, ref)
    err = rel_frob(out.data, ref.data)
    berr = block_errors(out, ref)
    print(f"D={D}: split vs FP64 oracle rel Frobenius {err:.3e}, worst block {berr.max():.3e}")
    assert err <= TOL
    assert berr.max() <= TOL_BLOCK


def test_split_steps_vs_oracle(gpu):
    lenv, psi, mpo1, mpo2, renv = workloads.heisenberg(800, 10, 3.0, 3)
    t1, _ = oracle.contract(lenv, psi, [[0], [0]])
    t2, _ = oracle.contract(t1, mpo1, [[0, 2], [0, 1]])
    t3, _ = oracle.contract(t2, mpo2, [[4, 1], [0, 1]])
    o, _ = oracle.contract(t3, renv, [[4, 1], [1, 0]])
    for a, b, ax, ref in ((lenv, psi, [[0], [0]], t1), (t3, renv, [[4, 1], [1, 0]], o)):
        plan = ContractionPlan(a, b, ax)
        c = plan.execute(DTensor.from_host(a), DTensor.from_host(b), mode="split")
        plan.device_status()
        assert rel_frob(c.to_host().data, ref.data) <= TOL


def test_split_wide_dynamic_range(gpu):
    """Rows and columns spanning 1e-150..1e150: the per-row/column power-of-two scales keep
    the relative error (scaled by the row and column maxima)."""
    a, b = workloads.config1(5)
    rng = np.random.default_rng(7)
    ra = 10.0 ** rng.uniform(-150, 150, size=a.shape()[0])
    # scale A's rows (leg 0) block by block
    starts = np.concatenate([[0], np.cumsum(a.legs[0].dims)[:-1]])
    data = a.data.copy()
    for blk in range(a.nblk):
        s = int(starts[a.coords[blk, 0]])
        shp = a.block_shapes()[blk]
        o = int(a.offsets[blk])
        view = data[o:o + int(np.prod(shp))].reshape(shp)
        view *= ra[s:s + shp[0], None, None]
    a2 = BSTensor(a.legs, a.coords, np.float64, data)
    ref, _ = oracle.contract(a2, b, [[2], [0]])
    plan = ContractionPlan(a2, b, [[2], [0]])
    c = plan.execute(DTensor.from_host(a2), DTensor.from_host(b), mode="split").to_host()
    # compare row by row (each output row carries one A-row scale)
    for blk in range(ref.nblk):
        x, y = c.block(blk), ref.block(blk)
        for i in range(y.shape[0]):
            n = np.linalg.norm(y[i])
            if n > 0:
                assert np.linalg.norm(x[i] - y[i]) / n <= 1e-11


def test_split_nonfinite(gpu):
    """NaN and infinities in A and B: every output they reach is non-finite (NaN from the
    tensor-core path, where FP64 gives NaN or an infinity), every other output within the bar."""
    a, b = workloads.config1(5)
    rng = np.random.default_rng(9)
    ad, bd = a.data.copy(), b.data.copy()
    ad[rng.choice(ad.size, 3, replace=False)] = [np.nan, np.inf, -np.inf]
    bd[rng.choice(bd.size, 2, replace=False)] = [np.inf, np.nan]
    a2 = BSTensor(a.legs, a.coords, np.float64, ad)
    b2 = BSTensor(b.legs, b.coords, np.float64, bd)
    outs = {}
    for mode in ("fp64", "split"):
        plan = ContractionPlan(a2, b2, [[2], [0]])
        with np.errstate(invalid="ignore", over="ignore"):
            outs[mode] = plan.execute(DTensor.from_host(a2), DTensor.from_host(b2), mode=mode).to_host().data
        plan.device_status()
    fin = np.isfinite(outs["fp64"])
    assert (~fin).any() and fin.any()
    assert np.array_equal(np.isfinite(outs["split"]), fin)
    x, y = outs["split"][~fin], outs["fp64"][~fin]
    assert (np.isnan(x) | (x == y)).all()   # skinny blocks run FP64 rows there: exact
    assert rel_frob(outs["split"][fin], outs["fp64"][fin]) <= TOL


@pytest.mark.parametrize("mode", ["fp64", "split"])
def test_matvec_apply_host(gpu, mode):
    """Host-buffer matvec (page-locked psi copied in, the result copied out) gives exactly the
    device-buffer result; an unpinned buffer is refused."""
    import torch
    from tensortoolkit_gb300 import capi
    lenv, psi, mpo1, mpo2, renv = workloads.heisenberg(800, 10, 3.0, 3)
    dl, d1, d2, dr = (DTensor.from_host(x) for x in (lenv, mpo1, mpo2, renv))
    mv = Matvec(dl, psi, d1, d2, dr, mode=mode)
    ref = mv.apply(DTensor.from_host(psi)).to_host()
    h_in = torch.from_numpy(psi.raw_f64()).pin_memory()
    h_out = torch.full((mv.result.size,), float("nan"), dtype=torch.float64).pin_memory()
    for _ in range(2):
        mv.apply_host(h_in, h_out)
    torch.cuda.synchronize()
    assert np.array_equal(h_out.numpy(), ref.data)
    with pytest.raises((capi.QltgError, ValueError)):
        mv.apply_host(h_in, torch.empty(mv.result.size, dtype=torch.float64))


@pytest.mark.parametrize("D", [1500, 6000])
def test_split_complex_fermionic_matvec_vs_oracle(gpu, D):
    """Split precision on complex operands (fU(1)xU(1) Hubbard-like chain, complex128): each
    complex GEMM runs as the real product of A's interleaved parts with B's 2 x 2 real form."""
    lenv, psi, mpo1, mpo2, renv = workloads.hubbard(D)
    ref, _ = oracle.matvec(lenv, psi, mpo1, mpo2, renv)
    dl, d1, d2, dr = (DTensor.from_host(x) for x in (lenv, mpo1, mpo2, renv))
    mv = Matvec(dl, psi, d1, d2, dr, mode="split")
    out = mv.apply(DTensor.from_host(psi))
    mv.device_status()
    out = out.to_host()
    assert same_topology(out, ref)
    err = rel_frob(out.data, ref.data)
    print(f"complex D={D}: split vs FP64 oracle rel Frobenius {err:.3e}")
    assert err <= TOL
