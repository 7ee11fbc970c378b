"""Pins the CPU oracle to the reference: the numpy restatement reproduces the
golden outputs of QSpace's own contractQS / permuteQS (compiled unmodified
behind the fake MATLAB runtime, tests/golden/make_golden.py) -- labels,
block order and itags exactly, data to FP rounding.  When the reference
oracle is built here (oracle/_ref), the restatement is also compared with
it on fresh seeded inputs."""
import json
from pathlib import Path

import numpy as np
import pytest

from oracle import qs_oracle as orc
from tests.golden.golden_io import unpack
from tests.helpers import assert_qspace_close

G = Path(__file__).resolve().parent / "golden"


def _cases(fname):
    z = np.load(G / fname)
    return z, json.loads(str(z["cases"]))


def test_oracle_matches_reference_contractQS():
    z, cases = _cases("contract_golden.npz")
    assert len(cases) >= 25
    for c in cases:
        n = c["name"]
        A, B, R = unpack(f"{n}_A", z), unpack(f"{n}_B", z), unpack(f"{n}_C", z)
        O = orc.contract(A, c["ia"], B, c["ib"], c["perm"])
        assert_qspace_close(O, R, 1e-14)
        if R["info"].get("itags"):
            assert O["info"].get("itags") == R["info"]["itags"], n


def test_oracle_matches_reference_permuteQS():
    z, cases = _cases("permute_golden.npz")
    for c in cases:
        n = c["name"]
        A, R = unpack(f"{n}_A", z), unpack(f"{n}_B", z)
        O = orc.permute(A, c["perm"], c["conj"])
        assert_qspace_close(O, R, 0.0)


def test_golden_has_edge_cases():
    _, cases = _cases("contract_golden.npz")
    names = {c["name"] for c in cases}
    for want in ("zero_rank3", "zero_rank2_herm", "numeric_idx", "autoconj", "case6_00", "case7_11"):
        assert want in names


def test_oracle_vs_live_reference_fresh_inputs():
    from oracle import ref
    if not ref.available("contractQS"):
        pytest.skip("reference oracle not built here (oracle/_ref)")
    from qspace_gb300.workloads import mps_site_tensor
    for seed in (0, 3, 4):
        A = mps_site_tensor(seed).to_dict()
        assert_qspace_close(orc.contract(A, "12*", A, "12"), ref.contractQS(A, "12*", A, "12"), 1e-14)
        # next site: its left leg carries the name of A's right leg
        B = mps_site_tensor(seed + 10).to_dict()
        B["info"] = {"itags": ["R", "s2", "X*"]}
        for ia, ib, perm in (("3", "1", "3,1,2,4"), ("3*", "1", None), ("1,3", "3,1", None)):
            if ia == "1,3":
                B2 = dict(B, info={"itags": ["R", "s2", "L*"]})
                R, O = ref.contractQS(A, ia, B2, ib, perm), orc.contract(A, ia, B2, ib, perm)
            else:
                R, O = ref.contractQS(A, ia, B, ib, perm), orc.contract(A, ia, B, ib, perm)
            assert_qspace_close(O, R, 1e-14)
            assert O["info"].get("itags") == R["info"].get("itags")


def _cell_items(z, c):
    return [x if x == "*" else unpack(f"{c['name']}_{x}", z) for x in c["items"]]


def test_oracle_matches_reference_cell_contractions():
    z, cases = _cases("cell_golden.npz")
    assert len(cases) >= 15
    for c in cases:
        R = unpack(f"{c['name']}_C", z)
        O = orc.contract_cell(_cell_items(z, c), c["perm"])
        assert_qspace_close(O, R, 1e-14)
        assert (O["info"].get("itags") or None) == (R["info"].get("itags") or None), c["name"]
