"""GEMM schedules and the tuner.

Bar: every selectable schedule gives the reference's result - FP64 tiles of 32 x 32 and
64 x 32, split precision with row stacking on and off - on the reference-written contraction
fixtures (real and fermionic complex) and on the matvec steps against the oracle: block
topology identical, values within 1e-12 relative Frobenius. The tuner picks one of the
candidates, records its timings, and a second plan with the same block structure takes the
choice from the cache without timing."""
import numpy as np
import pytest

from oracle import oracle
from tensortoolkit_gb300 import workloads
from tensortoolkit_gb300.api import ContractionPlan, DTensor, Matvec
from tensortoolkit_gb300.tensor import BSTensor, rel_frob, same_topology

pytestmark = pytest.mark.gpu

TOL = 1e-12
CASES = [("cfg1", ["c"]), ("matvec_u1_small", ["s1", "s2", "s3", "s4"]),
         ("ctrct_misc_u1", ["u_scalar", "u_perm", "u_mid", "f_env", "f_in", "f_mpo", "f_rev"]),
         ("matvec_f_small", ["s1", "s2", "s3", "s4"])]
SCHEDULES = [("fp64", dict(f64_tile_rows=32)), ("fp64", dict(f64_tile_rows=64)),
             ("split", dict(split_stack=1)), ("split", dict(split_stack=0))]


@pytest.mark.parametrize("mode,sched", SCHEDULES)
@pytest.mark.parametrize("case,tags", CASES)
def test_schedule_golden(gpu, golden, case, tags, mode, sched):
    rec = golden(case)
    for tag in tags:
        a = BSTensor.from_record(rec, tag + ".A")
        b = BSTensor.from_record(rec, tag + ".B")
        ref = BSTensor.from_record(rec, tag + ".C")
        ax = rec[tag + ".axes"]
        n = len(ax) // 2
        plan = ContractionPlan(a, b, [list(ax[:n]), list(ax[n:])])
        plan.set_schedule(**sched)
        c = plan.execute(DTensor.from_host(a), DTensor.from_host(b), mode=mode)
        plan.device_status()
        c = c.to_host()
        if ref.rank:
            assert same_topology(c, ref)
        assert rel_frob(c.data, ref.data) <= TOL, (case, tag, mode, sched)


@pytest.mark.parametrize("mode,sched", SCHEDULES)
@pytest.mark.parametrize("kind", ["u1", "fermionic"])
def test_schedule_matvec_steps(gpu, kind, mode, sched):
    """The four matvec contractions, chained on the device, against the oracle chain."""
    if kind == "u1":
        lenv, psi, mpo1, mpo2, renv = workloads.heisenberg(1200, 12, 4.0, 2)
    else:
        lenv, psi, mpo1, mpo2, renv = workloads.hubbard(900, 6, 5)
    ref, _ = oracle.matvec(lenv, psi, mpo1, mpo2, renv)
    axes = [[[0], [0]], [[0, 2], [0, 1]], [[4, 1], [0, 1]], [[4, 1], [1, 0]]]
    cur, meta = DTensor.from_host(lenv), lenv
    for i, b in enumerate((psi, mpo1, mpo2, renv)):
        plan = ContractionPlan(meta, b, axes[i])
        plan.set_schedule(**sched)
        cur = plan.execute(cur, DTensor.from_host(b), mode=mode)
        plan.device_status()
        meta = plan.result
    out = cur.to_host()
    assert same_topology(out, ref)
    assert rel_frob(out.data, ref.data) <= TOL, (kind, mode, sched)


def test_stacking_reduces_padding(gpu):
    """At D=4000 the first matvec step's stacked schedule executes fewer padded tile stages."""
    lenv, psi, *_ = workloads.heisenberg(4000, 30, 9.0, 1)
    stats = {}
    for stack in (0, 1):
        plan = ContractionPlan(lenv, psi, [[0], [0]])
        plan.set_schedule(split_stack=stack)
        plan.execute(DTensor.from_host(lenv), DTensor.from_host(psi), mode="split")
        plan.device_status()
        stats[stack] = plan.split_stats()
    print("tile stages / useful share, unstacked:", stats[0], "stacked:", stats[1])
    assert stats[1][0] < stats[0][0] and stats[1][1] > stats[0][1]


@pytest.mark.parametrize("mode", ["fp64", "split"])
def test_tuner_choice_and_cache(gpu, mode):
    lenv, psi, *_ = workloads.heisenberg(2000, 20, 6.0, 1)
    dl, dp = DTensor.from_host(lenv), DTensor.from_host(psi)
    p1 = ContractionPlan(lenv, psi, [[0], [0]])
    cached_first = p1.tune(dl, dp, mode=mode)
    s1 = p1.schedule()
    assert s1["tuned"][mode]
    chosen, slowest = s1["tuned_ms"][mode]
    if not cached_first:
        assert 0 < chosen <= slowest
    ref = p1.execute(dl, dp, mode=mode).to_host()
    # same block structure: the cached choice, no timing, the same result
    p2 = ContractionPlan(lenv, psi, [[0], [0]])
    assert p2.tune(dl, dp, mode=mode)
    s2 = p2.schedule()
    assert (s2["f64_tile_rows"], s2["split_stack"]) == (s1["f64_tile_rows"], s1["split_stack"])
    out = p2.execute(dl, dp, mode=mode).to_host()
    assert np.array_equal(out.data, ref.data)


def test_matvec_records_tuned_schedules(gpu):
    lenv, psi, mpo1, mpo2, renv = workloads.heisenberg(800, 10, 3.0, 3)
    dl, d1, d2, dr = (DTensor.from_host(x) for x in (lenv, mpo1, mpo2, renv))
    for mode in ("fp64", "split"):
        mv = Matvec(dl, psi, d1, d2, dr, mode=mode)
        sch = mv.schedules()
        # steps 0 and 3 have tiles to schedule; the MPO steps are skinny-only
        assert sch[0]["tuned"][mode] and sch[3]["tuned"][mode]
        if mode == "split":
            assert sch[0]["split_tile_stages"] > 0 and 0 < sch[0]["split_useful_frac"] <= 1
