"""Reusable grouped plans (qs_grouped_plan_*): a plan replayed as a CUDA graph
gives the one-shot entry point's result on every run (bit for bit with the
same digit plan), re-records when the buffers change, and the autotuner picks
a digit width that meets the tolerance and is remembered for the shape."""
import numpy as np
import pytest

from qspace_gb300.grouped import DeviceBatch, Packed
from qspace_gb300.workloads import grouped_pairs

pytestmark = pytest.mark.gpu


def _rel(C, R):
    num = sum(float(np.sum(np.abs(c - r) ** 2)) for c, r in zip(C, R))
    den = sum(float(np.sum(np.abs(r) ** 2)) for r in R)
    return np.sqrt(num / den)


def _batch(ctx, seed=3, n=60, cplx=True, blk=None):
    w = grouped_pairs(seed=seed, npairs=n, lo=4, hi=400, complex_data=cplx)
    return DeviceBatch(Packed(w["A"], w["B"], w["afac"], blk=blk, cplx=cplx), ctx)


def _poison(db):
    db.dC.fill_(float("nan"))


@pytest.mark.parametrize("prec", ["fp64", "split"])
@pytest.mark.parametrize("cplx", [False, True])
def test_plan_replays_match_one_shot(ctx, prec, cplx):
    db = _batch(ctx, cplx=cplx)
    db.run(prec)
    ref = [c.copy() for c in db.result()]
    plan = db.plan(prec)
    launches = []
    for _ in range(3):
        _poison(db)
        st = {}
        db.run_plan(plan, st)
        launches.append(st["launches"])
        got = db.result()
        for g, r in zip(got, ref):
            assert np.array_equal(g, r)
    # first run launches directly (and records); the replays count the graph's kernels
    assert launches[0] >= 1 and launches[1] == launches[2] == launches[0]
    plan.close()


def test_plan_rerecords_for_new_buffers(ctx):
    import torch
    db = _batch(ctx, seed=4, n=30)
    db.run("split")
    ref = [c.copy() for c in db.result()]
    plan = db.plan("split")
    db.run_plan(plan)
    C1 = db.dC
    C2 = torch.full_like(C1, float("nan"))
    for buf in (C2, C1, C2):
        db.dC = buf
        _poison(db)
        db.run_plan(plan)
        assert all(np.array_equal(g, r) for g, r in zip(db.result(), ref))
    db.dC = C1
    plan.close()


def test_plan_without_graph(ctx):
    db = _batch(ctx, seed=5, n=20, cplx=False)
    db.run("fp64")
    ref = [c.copy() for c in db.result()]
    plan = db.plan("fp64", graph=False)
    _poison(db)
    db.run_plan(plan)
    assert all(np.array_equal(g, r) for g, r in zip(db.result(), ref))
    plan.close()


def test_autotune_meets_tolerance_and_is_remembered(ctx):
    db = _batch(ctx, seed=6, n=80)
    db.run("fp64")
    exact = [c.copy() for c in db.result()]
    p1 = db.plan("split", autotune=True)
    st1 = {}
    _poison(db)
    db.run_plan(p1, st1)
    assert st1["digit_bits"] in (5, 6, 7, 8) and st1["device_ms"] > 0
    assert _rel(db.result(), exact) <= 1e-12
    _poison(db)
    db.run_plan(p1)               # replay of the tuned plan
    assert _rel(db.result(), exact) <= 1e-12
    # a second plan over the same shapes reuses the choice without timing
    p2 = db.plan("split", autotune=True)
    st2 = {}
    _poison(db)
    db.run_plan(p2, st2)
    assert st2["digit_bits"] == st1["digit_bits"] and st2["device_ms"] == 0
    assert _rel(db.result(), exact) <= 1e-12
    p1.close()
    p2.close()


def test_plan_shared_output_blocks(ctx):
    # four pairs of different depth summing into one 50 x 70 block
    rng = np.random.default_rng(9)
    A = [np.asfortranarray(rng.standard_normal((50, k))) for k in (10, 200, 33, 1)]
    B = [np.asfortranarray(rng.standard_normal((k, 70))) for k in (10, 200, 33, 1)]
    afac = rng.uniform(-1, 1, 4)
    pk = Packed(A, B, afac, blk=[0, 0, 0, 0], cplx=False)
    db = DeviceBatch(pk, ctx)
    plan = db.plan("split")
    db.run_plan(plan)
    db.run_plan(plan)
    exact = sum(f * (a @ b) for a, b, f in zip(A, B, afac))
    got = db.result()[0]
    assert np.linalg.norm(got - exact) <= 1e-12 * np.linalg.norm(exact)
    plan.close()
