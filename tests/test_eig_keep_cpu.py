"""eigQS's truncation (markSet over all blocks' eigenvalues: Nkeep, Etrunc,
degeneracy averaging with the weighted-gap cut for deps > 0) against fixtures
made by the REFERENCE's own eigQS (tests/golden/make_eig_golden.py): the
oracle's restatement and the library's host implementation (qs_mark_keep)
keep the same states of every sector as the reference and report the same NK
(with Etrunc > 0 and deps = 0 the reference's NK stays min(Nkeep, N) while
its kept set EK follows Etrunc)."""
import json
from pathlib import Path

import numpy as np
import pytest

from oracle import qs_oracle as orc
from qspace_gb300.linalg import mark_keep
from tests.golden.golden_io import unpack

G = Path(__file__).resolve().parent / "golden"


def _cases():
    z = np.load(G / "eig_golden.npz")
    return z, json.loads(str(z["cases"]))


@pytest.mark.parametrize("impl", ["oracle", "library"])
def test_eig_truncation_matches_reference(impl):
    z, cases = _cases()
    assert len(cases) == 10
    for c in cases:
        H, EK = unpack(f"{c['name']}_H", z), unpack(f"{c['name']}_EK", z)
        E = [np.linalg.eigvalsh(np.asarray(d)) for d in H["data"]]
        o = c["opts"]
        args = (int(o.get("Nkeep", -1)), float(o.get("Etrunc", 0.0)), float(o.get("deps", 0.0)))
        if impl == "oracle":
            keep, nk = orc.mark_keep(E, *args)
        else:
            keep, nk, _ = mark_keep(E, *args)
        assert nk == c["NK"], c
        assert sum(int(np.sum(k)) for k in keep) == sum(np.size(d) for d in EK["data"]), c
        got = {tuple(np.asarray(H["Q"][0][i]).ravel()): E[i][np.asarray(keep[i], bool)] for i in range(len(E))
               if np.any(keep[i])}
        ref = {tuple(np.asarray(EK["Q"][0][i]).ravel()): np.sort(np.asarray(d).ravel()) for i, d in enumerate(EK["data"])}
        assert got.keys() == ref.keys(), c["name"]
        for k in ref:
            assert np.allclose(got[k], ref[k], rtol=1e-12, atol=1e-12), (c["name"], k)
