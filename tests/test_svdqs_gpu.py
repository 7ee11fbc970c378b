"""svdQS end to end with the block SVD on the GPU (qs_svd_blocks_ex) against
the fixtures made by the REFERENCE's own svdQS, and on larger two-site
wavefunctions against LAPACK's SVD of the same block matrices."""
import json
from pathlib import Path

import numpy as np
import pytest

from qspace_gb300.linalg import _SvdLayout, svdQS
from qspace_gb300.qspace import QSpace
from qspace_gb300.workloads import two_site_state
from tests.golden.golden_io import unpack
from tests.helpers import assert_svd_matches

pytestmark = pytest.mark.gpu

G = Path(__file__).resolve().parent / "golden"
Z = np.load(G / "svdqs_golden.npz")
CASES = json.loads(str(Z["cases"]))


def _opts(o):
    return dict(Nkeep=o.get("Nkeep", -1), Nkmin=o.get("Nkmin", 0), stol=o.get("stol"), itag=o.get("itag", ""),
                permA=o.get("permA"), permB=o.get("permB"))


@pytest.mark.parametrize("case", CASES, ids=[c["name"] for c in CASES])
def test_svdqs_matches_reference(ctx, case):
    A = QSpace.from_dict(unpack(f"{case['name']}_A", Z))
    if case.get("error"):
        with pytest.raises(ValueError):
            svdQS(A, case["idx"], ctx=ctx, **_opts(case["opts"]))
        return
    U, S, V, info = svdQS(A, case["idx"], ctx=ctx, **_opts(case["opts"]))
    ref = [unpack(f"{case['name']}_{t}", Z) for t in "USV"]
    assert_svd_matches((U, S, V), ref, case["idx"], case["opts"], tol=1e-11)
    assert info["Nkeep"] == case["Nkeep"] and info["flag"] == case["flag"]
    assert abs(info["sfac"] - case["sfac"]) <= 1e-12 * case["sfac"]
    assert np.allclose(info["svd"], Z[f"{case['name']}_svd"], rtol=1e-12, atol=1e-13)


def _two_site(seed, D, cplx):
    return two_site_state(seed, D, cplx)


@pytest.mark.parametrize("cplx", [False, True])
@pytest.mark.parametrize("idx,opts", [([3, 4], {"Nkeep": 200}), ([4], {}), ([2, 3, 4], {"stol": 1e-3})])
def test_svdqs_two_site_against_lapack(ctx, cplx, idx, opts):
    A = _two_site(11, 96, cplx)
    U, S, V, info = svdQS(A, idx, ctx=ctx, **_opts(opts))
    L = _SvdLayout(A, idx)
    dec = [np.linalg.svd(M, full_matrices=False) for M in L.mats]
    ref = L.finish([d[0] for d in dec], [d[1] for d in dec], [d[2] for d in dec], **_opts(opts))
    assert_svd_matches((U, S, V), [x.to_dict() for x in ref[:3]], idx, opts, tol=1e-11)
    assert info["Nkeep"] == ref[3]["Nkeep"] and abs(info["sfac"] - ref[3]["sfac"]) <= 1e-12


OCASES = json.loads(str(Z["ortho_cases"]))


@pytest.mark.parametrize("case", OCASES, ids=[c["name"] for c in OCASES])
def test_orthoqs_matches_reference(ctx, case):
    from qspace_gb300.linalg import _OrthoPlan, orthoQS
    from tests.helpers import assert_ortho_matches
    from tests.test_orthoqs_cpu import bonds
    A = QSpace.from_dict(unpack(f"{case['name']}_A", Z))
    o = case["opts"]
    kw = dict(Nkeep=o.get("Nkeep", -1), Nkmin=o.get("Nkmin", 0), stol=o.get("stol"), itag=o.get("itag", ""),
              permA=o.get("permA"), permB=o.get("permB"), ctx=ctx)
    if case.get("error"):
        with pytest.raises(ValueError):
            orthoQS(A, case["idx"], case["lrdir"], **kw)
        return
    A1, A2, info = orthoQS(A, case["idx"], case["lrdir"], **kw)
    ref = [unpack(f"{case['name']}_{t}", Z) for t in ("A1", "A2")]
    pl = _OrthoPlan(A, case["idx"], case["lrdir"], o.get("permA"), o.get("permB"))
    if A1.nblk:
        assert_ortho_matches((A1, A2), ref, *bonds(pl, A1, A2), tol=1e-11, iso=2 if pl.swap else 1)
    else:
        assert not ref[0]["data"]
    assert info["Nkeep"] == case["Nkeep"] and info["flag"] == case["flag"]
