"""The CUDA path against the REFERENCE's own outputs (golden fixtures made by
QSpace's contractQS / permuteQS, tests/golden/make_golden.py): labels, block
order and itags bit-exact; data within 1e-14 (plain FP64 path) and 1e-12
(split BF16 path) relative Frobenius error."""
import json
from pathlib import Path

import numpy as np
import pytest

from qspace_gb300 import QSpace, contractQS, permuteQS
from tests.golden.golden_io import unpack
from tests.helpers import assert_qspace_close

pytestmark = pytest.mark.gpu
G = Path(__file__).resolve().parent / "golden"


def _cases(fname):
    z = np.load(G / fname)
    return z, json.loads(str(z["cases"]))


@pytest.mark.parametrize("prec,tol", [("fp64", 1e-14), ("split", 1e-12)])
def test_contractQS_matches_reference(ctx, prec, tol):
    z, cases = _cases("contract_golden.npz")
    for c in cases:
        n = c["name"]
        A, B, R = unpack(f"{n}_A", z), unpack(f"{n}_B", z), unpack(f"{n}_C", z)
        C = contractQS(QSpace.from_dict(A), c["ia"], QSpace.from_dict(B), c["ib"], c["perm"], prec=prec, ctx=ctx)
        assert_qspace_close(C, R, tol)
        assert C.info.get("itags") == R["info"].get("itags"), n


def test_permuteQS_matches_reference(ctx):
    z, cases = _cases("permute_golden.npz")
    for c in cases:
        n = c["name"]
        A, R = unpack(f"{n}_A", z), unpack(f"{n}_B", z)
        B = permuteQS(QSpace.from_dict(A), c["perm"], c["conj"], ctx=ctx)
        assert_qspace_close(B, R, 0.0)
        assert B.info.get("itags") == R["info"].get("itags"), n


@pytest.mark.parametrize("prec,tol", [("fp64", 1e-14), ("split", 1e-12)])
def test_cell_contraction_matches_reference(ctx, prec, tol):
    from qspace_gb300 import contract_itags, upload
    z, cases = _cases("cell_golden.npz")
    for c in cases:
        items = [x if x == "*" else QSpace.from_dict(unpack(f"{c['name']}_{x}", z)) for x in c["items"]]
        R = unpack(f"{c['name']}_C", z)
        C = contract_itags(items, c["perm"], prec=prec, ctx=ctx)
        assert_qspace_close(C, R, tol)
        assert (C.info.get("itags") or None) == (R["info"].get("itags") or None), c["name"]
        # the same chain on device-resident tensors
        dev = [x if x == "*" else upload(x, ctx) for x in items]
        Cd = contract_itags(dev, c["perm"], prec=prec).download()
        assert_qspace_close(Cd, R, tol)
