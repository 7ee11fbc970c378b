"""The batched grouped contraction at its full size: 2000 complex128 block
pairs, M, N, K log-uniform in [8, 1024], a CG factor per pair, seed 0 (the
workload the throughput figure is quoted on).  Every pair of the batch is
checked against numpy's FP64 product afac_p * A_p @ B_p:

* split BF16 path through the one-shot entry point (qs_grouped_gemm) and
  through a reusable plan with the autotuned digit width (the timed path):
  relative Frobenius error over all pairs <= 1e-12, and no single pair above
  1e-12 either;
* plain FP64 path: <= 1e-14 over all pairs.
"""
import numpy as np
import pytest

from qspace_gb300.grouped import DeviceBatch, Packed
from qspace_gb300.workloads import grouped_pairs

pytestmark = pytest.mark.gpu

SPLIT_TOL = 1e-12
FP64_TOL = 1e-14


@pytest.fixture(scope="module")
def full(ctx):
    w = grouped_pairs(seed=0, npairs=2000, complex_data=True)
    ref = [w["afac"][p] * (w["A"][p] @ w["B"][p]) for p in range(2000)]
    db = DeviceBatch(Packed(w["A"], w["B"], w["afac"], cplx=True), ctx)
    del w
    yield db, ref
    del db


def _errors(C, R):
    num = np.array([float(np.sum(np.abs(c - r) ** 2)) for c, r in zip(C, R)])
    den = np.array([float(np.sum(np.abs(r) ** 2)) for r in R])
    return float(np.sqrt(num.sum() / den.sum())), float(np.sqrt(np.max(num / den)))


def test_full_size_split_one_shot(full):
    db, ref = full
    db.dC.fill_(float("nan"))
    st = {}
    db.run("split", stats=st)
    tot, worst = _errors(db.result(), ref)
    assert st["nslices"] >= 5
    assert tot <= SPLIT_TOL, tot
    assert worst <= SPLIT_TOL, worst


def test_full_size_split_autotuned_plan(full):
    db, ref = full
    plan = db.plan("split", autotune=True)
    for _ in range(2):          # the tuning run, then a graph replay
        db.dC.fill_(float("nan"))
        db.run_plan(plan)
        tot, worst = _errors(db.result(), ref)
        assert tot <= SPLIT_TOL, tot
        assert worst <= SPLIT_TOL, worst
    plan.close()


def test_full_size_plain_fp64(full):
    db, ref = full
    db.dC.fill_(float("nan"))
    db.run("fp64")
    tot, worst = _errors(db.result(), ref)
    assert tot <= FP64_TOL, tot
