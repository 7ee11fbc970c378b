"""The QSpace-level orthoQS (usages #1 and #2) against fixtures made by the
REFERENCE's own orthoQS (tests/golden/make_svdqs_golden.py): the host side
of the product (which legs lead, the block matrices, the truncation with the
reference's Nkeep estimate, A1 = U and A2 = V S with their labels, block
order, itags and the lrdir / permA / permB permutations) fed with LAPACK's
SVD of the same block matrices, so that this runs without a GPU."""
import json
from pathlib import Path

import numpy as np
import pytest

from qspace_gb300.linalg import _OrthoPlan
from qspace_gb300.qspace import QSpace
from tests.golden.golden_io import unpack
from tests.helpers import assert_ortho_matches

G = Path(__file__).resolve().parent / "golden"
Z = np.load(G / "svdqs_golden.npz")
CASES = json.loads(str(Z["ortho_cases"]))


def bonds(plan, A1, A2):
    """Leg of the new bond in A1 and A2: last in U and in V S before the
    final permutations pa / pb."""
    r1, r2 = A1.rank, A2.rank
    return (plan.pa.index(r1 - 1) if plan.pa is not None else r1 - 1), plan.pb.index(r2 - 1)


def host_ortho(A, case):
    o = case["opts"]
    pl = _OrthoPlan(QSpace.from_dict(A), case["idx"], case["lrdir"], o.get("permA"), o.get("permB"))
    dec = [np.linalg.svd(M, full_matrices=False) for M in pl.L.mats]
    A1, A2, info = pl.finish([d[0] for d in dec], [d[1] for d in dec], [d[2] for d in dec], o.get("Nkeep", -1),
                             o.get("Nkmin", 0), o.get("stol"), o.get("itag", ""))
    return pl, A1, A2, info


def test_fixture_inventory():
    assert len(CASES) == 17
    assert sum(1 for c in CASES if c.get("error")) == 1
    assert {c["lrdir"] for c in CASES} >= {None, ">>", "<<", "LR", "RL", "+", "-"}


@pytest.mark.parametrize("case", CASES, ids=[c["name"] for c in CASES])
def test_orthoqs_host_matches_reference(case):
    A = unpack(f"{case['name']}_A", Z)
    if case.get("error"):
        with pytest.raises(ValueError):
            host_ortho(A, case)
        return
    pl, A1, A2, info = host_ortho(A, case)
    ref = [unpack(f"{case['name']}_{t}", Z) for t in ("A1", "A2")]
    if A1.nblk:
        assert_ortho_matches((A1, A2), ref, *bonds(pl, A1, A2), tol=1e-12, iso=2 if pl.swap else 1)
    else:
        assert not ref[0]["data"] and not ref[1]["data"]
    assert info["Nkeep"] == case["Nkeep"] and info["flag"] == case["flag"]
    assert abs(info["sfac"] - case["sfac"]) <= 1e-13 * case["sfac"]
