"""The QSpace-level svdQS against fixtures made by the REFERENCE's own svdQS
(tests/golden/make_svdqs_golden.py): the host side of the product (grouping
of PSI's blocks into one matrix per conserved label sum, the truncation, the
U / S / Vd QSpaces with their labels, block order, itags and permutations)
fed with LAPACK's SVD of the same block matrices, so that this runs without
a GPU.  Rejected inputs raise like the reference."""
import json
from pathlib import Path

import numpy as np
import pytest

from qspace_gb300.linalg import _SvdLayout
from qspace_gb300.qspace import QSpace
from tests.golden.golden_io import unpack
from tests.helpers import assert_svd_matches

G = Path(__file__).resolve().parent / "golden"
Z = np.load(G / "svdqs_golden.npz")
CASES = json.loads(str(Z["cases"]))


def _host_svdqs(A, idx, opts):
    L = _SvdLayout(QSpace.from_dict(A), idx)
    Us, Ss, Vts = [], [], []
    for M in L.mats:
        u, s, vt = np.linalg.svd(M, full_matrices=False)
        Us.append(u)
        Ss.append(s)
        Vts.append(vt)
    return L.finish(Us, Ss, Vts, Nkeep=opts.get("Nkeep", -1), Nkmin=opts.get("Nkmin", 0), stol=opts.get("stol"),
                    itag=opts.get("itag", ""), permA=opts.get("permA"), permB=opts.get("permB"))


def test_fixture_inventory():
    assert len(CASES) == 28
    assert sum(1 for c in CASES if c.get("error")) == 2
    assert any(c.get("Nkeep") == 0 for c in CASES)


@pytest.mark.parametrize("case", CASES, ids=[c["name"] for c in CASES])
def test_svdqs_host_matches_reference(case):
    A = unpack(f"{case['name']}_A", Z)
    if case.get("error"):
        with pytest.raises(ValueError):
            _host_svdqs(A, case["idx"], case["opts"])
        return
    U, S, V, info = _host_svdqs(A, case["idx"], case["opts"])
    ref = [unpack(f"{case['name']}_{t}", Z) for t in "USV"]
    assert_svd_matches((U, S, V), ref, case["idx"], case["opts"], tol=1e-12)
    assert info["Nkeep"] == case["Nkeep"] and info["Ntot"] == case["Ntot"] and info["flag"] == case["flag"]
    assert abs(info["sfac"] - case["sfac"]) <= 1e-13 * case["sfac"]
    assert abs(info["svd2tr"] - case["svd2tr"]) <= 1e-13
    assert np.allclose(info["svd"], Z[f"{case['name']}_svd"], rtol=1e-13, atol=1e-14)
