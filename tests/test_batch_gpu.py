"""Batched contractions (qs_contract_batch): the block products of many
contractions share one grouped launch per element type (and digit plan);
every result equals the same contraction run alone, bit for bit, on both the
FP64 and the split path, and the split results are within 1e-12 of FP64."""
import numpy as np
import pytest

from qspace_gb300 import contract_batch, contract_dev, upload
from qspace_gb300.workloads import mps_site_tensor, random_abelian, random_leg
from tests.helpers import assert_qspace_close

pytestmark = pytest.mark.gpu


def _jobs(ctx):
    rng = np.random.default_rng(31)
    t = [random_leg(rng, nsec=3, dmax=6, qdim=2) for _ in range(5)]
    jobs = []
    for seed, cx in ((0, False), (1, True), (2, False)):
        A = upload(mps_site_tensor(seed, D=256, complex_data=cx), ctx)
        jobs.append((A, "12*", A, "12", None))
    for cx in (False, True):
        A = upload(random_abelian(rng, [t[0], t[1], t[2]], complex_data=cx, itags=["a", "b", "c"]), ctx)
        B = upload(random_abelian(rng, [t[2], t[3], t[1]], complex_data=cx, itags=["c*", "d", "b*"]), ctx)
        jobs.append((A, "2,3", B, "3,1", [2, 1]))
        jobs.append((A, "3", B, "1", [4, 1, 3, 2]))
    # mixed real x complex (the real operand is widened)
    Ar = upload(random_abelian(rng, [t[0], t[1]], itags=["p", "q"]), ctx)
    Bz = upload(random_abelian(rng, [t[1], t[4]], complex_data=True, itags=["q*", "r"]), ctx)
    jobs.append((Ar, "2", Bz, "1", None))
    return jobs


@pytest.mark.parametrize("prec", ["fp64", "split"])
def test_batch_matches_single_calls(ctx, prec):
    jobs = _jobs(ctx)
    alone = [contract_dev(a, ia, b, ib, p, prec=prec).download() for (a, ia, b, ib, p) in jobs]
    exact = [contract_dev(a, ia, b, ib, p, prec="fp64").download() for (a, ia, b, ib, p) in jobs]
    l0 = ctx.launches
    got = contract_batch(jobs, prec=prec)
    batch_launches = ctx.launches - l0
    assert len(got) == len(jobs)
    for g, r, e in zip(got, alone, exact):
        G = g.download()
        assert G.info.get("itags") == r.info.get("itags")
        assert len(G.data) == len(r.data)
        for x, y in zip(G.data, r.data):
            assert np.array_equal(x, y)
        for k in range(len(G.Q)):
            assert np.array_equal(G.Q[k], r.Q[k])
        assert_qspace_close(G, e.to_dict(), 1e-12)
    l1 = ctx.launches
    for (a, ia, b, ib, p) in jobs:
        contract_dev(a, ia, b, ib, p, prec=prec)
    assert batch_launches < ctx.launches - l1


def test_batch_empty_and_single(ctx):
    assert contract_batch([]) == []
    A = upload(mps_site_tensor(4, D=128), ctx)
    (T,) = contract_batch([(A, "12*", A, "12")])
    R = contract_dev(A, "12*", A, "12").download()
    assert_qspace_close(T.download(), R.to_dict(), 0.0)
