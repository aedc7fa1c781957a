"""Split mode on the skinny output blocks (n, k <= 8: the MPO steps of the two-site matvec,
which run FP64 rows) and through the whole matvec, with special values, through the C ABI,
against FP64 (the GPU's FP64 mode and the oracle).

Bar: whole results within 1e-12 relative Frobenius of FP64; skinny steps element by element
within 2^-40 sum_k |a||b| of FP64 with NaN and infinity exactly where FP64 has them (rows with
non-finite, subnormal, tiny and huge entries, results leaving the FP64 range, B columns with a
subnormal or infinite entry, blocks stacking more than 8 contracted columns); the matvec
non-finite exactly where FP64 is."""
import itertools

import numpy as np
import pytest

from oracle import oracle
from tensortoolkit_gb300 import workloads
from tensortoolkit_gb300.api import ContractionPlan, DTensor, Matvec
from tensortoolkit_gb300.tensor import IN, OUT, BSTensor, Leg, rel_frob, same_topology

pytestmark = pytest.mark.gpu

ELEM_TOL = 2.0 ** -40


def _run(a, b, axes, mode):
    plan = ContractionPlan(a, b, axes)
    c = plan.execute(DTensor.from_host(a), DTensor.from_host(b), mode=mode)
    plan.device_status()
    return c.to_host()


def _abs(t: BSTensor) -> BSTensor:
    return BSTensor(t.legs, t.coords, np.float64, np.abs(t.data))


def _check_elementwise(a, b, axes, got, ref):
    """|got - ref| <= 2^-40 sum |a||b| where ref is finite; NaN / inf exactly where ref has them."""
    assert same_topology(got, ref)
    x, y = got.data, ref.data
    assert np.array_equal(np.isnan(x), np.isnan(y))
    inf = np.isinf(y)
    assert np.array_equal(np.isinf(x), inf) and np.array_equal(x[inf], y[inf])
    fin = np.isfinite(y)
    with np.errstate(invalid="ignore", over="ignore"):
        bound = _run(_abs(a), _abs(b), axes, "fp64").data
    bound = np.where(np.isfinite(bound), bound, np.inf)
    err = np.abs(x[fin] - y[fin])
    assert np.all(err <= ELEM_TOL * bound[fin] + 1e-300), float(np.max(err / (bound[fin] + 1e-300)))


@pytest.fixture(scope="module")
def mpo_step():
    """Step 1 of a D=800 matvec: t1 = lenv . psi contracted with mpo1 over (w, s1)."""
    lenv, psi, mpo1, _, _ = workloads.heisenberg(800, 10, 3.0, 3)
    t1, _ = oracle.contract(lenv, psi, [[0], [0]])
    return t1, mpo1, [[0, 2], [0, 1]]


def test_mpo_step_vs_oracle(gpu, mpo_step):
    a, b, axes = mpo_step
    ref, _ = oracle.contract(a, b, axes)
    got = _run(a, b, axes, "split")
    err = rel_frob(got.data, ref.data)
    assert same_topology(got, ref) and err <= 1e-12
    _check_elementwise(a, b, axes, got, _run(a, b, axes, "fp64"))


def test_mpo_step_special_rows(gpu, mpo_step):
    a, b, axes = mpo_step
    rng = np.random.default_rng(11)
    d = a.data.copy()
    n = d.size
    pos = rng.choice(n, size=60, replace=False)
    d[pos[:5]] = np.nan
    d[pos[5:10]] = np.inf
    d[pos[10:15]] = -np.inf
    d[pos[15:35]] = 1e-310                                   # subnormal entries
    d[pos[35:60]] = 0.0
    sh = a.block_shapes()
    for blk, scale in ((1, 1e-300), (2, 1e290), (3, 1e308)):  # tiny rows, big rows, overflow
        o, m = int(a.offsets[blk]), int(np.prod(sh[blk]))
        d[o:o + m] *= scale
    o, m = int(a.offsets[4]), int(np.prod(sh[4]))            # one block over 250 decades
    d[o:o + m] *= 10.0 ** rng.uniform(-250, 0, size=m)
    a2 = BSTensor(a.legs, a.coords, np.float64, d)
    with np.errstate(invalid="ignore", over="ignore"):
        ref = _run(a2, b, axes, "fp64")
    got = _run(a2, b, axes, "split")
    _check_elementwise(a2, b, axes, got, ref)


def test_mpo_step_special_columns(gpu, mpo_step):
    a, b, axes = mpo_step
    for special in (1e-310, np.inf, 1e-250):
        d = b.data.copy()
        d[np.flatnonzero(d)[3]] = special
        b2 = BSTensor(b.legs, b.coords, np.float64, d)
        with np.errstate(invalid="ignore", over="ignore"):
            ref = _run(a, b2, axes, "fp64")
        got = _run(a, b2, axes, "split")
        _check_elementwise(a, b2, axes, got, ref)


def _rand(legs, rng):
    sign = [1 if l.dir == OUT else -1 for l in legs]
    coords = [c for c in itertools.product(*[range(l.nsct) for l in legs])
              if sum(s * int(l.qns[ci, 0]) for s, l, ci in zip(sign, legs, c)) == 0]
    t = BSTensor(legs, np.array(coords, np.int64), np.float64)
    t.data = rng.standard_normal(t.size)
    return t


def test_stacked_extent_above_8(gpu):
    """Output blocks stacking 4, 8 and 12 contracted columns over 1 to 3 tasks."""
    rng = np.random.default_rng(5)
    L = Leg(IN, np.arange(0, 5), rng.integers(40, 400, size=5))
    p = Leg(OUT, np.arange(0, 3), np.full(3, 2))
    q = Leg(IN, np.arange(0, 5), np.array([1, 3, 2, 3, 1]))
    a = _rand([L, p, p], rng)
    b = _rand([p.inverse(), p.inverse(), q.inverse()], rng)
    axes = [[1, 2], [0, 1]]
    ref, _ = oracle.contract(a, b, axes)
    got = _run(a, b, axes, "split")
    assert same_topology(got, ref) and rel_frob(got.data, ref.data) <= 1e-12
    _check_elementwise(a, b, axes, got, _run(a, b, axes, "fp64"))


def test_matvec_specials(gpu):
    """One matvec applied to changing psi (operands sliced once stay valid), values over 60
    decades, then infinities, a NaN and a subnormal in psi."""
    lenv, psi, mpo1, mpo2, renv = workloads.heisenberg(600, 8, 3.0, 2)
    dl, d1, d2, dr = (DTensor.from_host(x) for x in (lenv, mpo1, mpo2, renv))
    mv = Matvec(dl, psi, d1, d2, dr, mode="split")
    rng = np.random.default_rng(3)
    for trial in range(3):
        p = psi.copy()
        p.data = rng.standard_normal(p.size) * 10.0 ** rng.uniform(-30, 30, size=p.size)
        if trial == 2:
            p.data[rng.choice(p.size, 4, replace=False)] = [np.inf, -np.inf, np.nan, 1e-310]
        with np.errstate(invalid="ignore", over="ignore"):
            ref, _ = oracle.matvec(lenv, p, mpo1, mpo2, renv)
        out = mv.apply(DTensor.from_host(p))
        mv.device_status()
        got = out.to_host()
        assert same_topology(got, ref)
        fin = np.isfinite(ref.data)
        # non-finite exactly where FP64 has it (the tensor-core steps store NaN for an
        # infinity: their slices cannot carry one), the rest within the split bar
        assert np.array_equal(np.isfinite(got.data), fin)
        if fin.any():
            assert rel_frob(got.data[fin], ref.data[fin]) <= 1e-12
