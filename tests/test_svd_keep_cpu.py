"""The truncation of svdQS (dmrgTruncate: markSet in descending order,
Nkeep / Nkmin / stol, norm-preserving rescale) against fixtures made by the
REFERENCE's own svdQS (tests/golden/make_svd_golden.py): the oracle's
restatement and the library's host implementation (qs_svd_keep) reproduce
the reference's kept count, rescale factor, discarded weight and the kept
singular values of every block."""
import ctypes as C
import json
from pathlib import Path

import numpy as np
import pytest

from oracle import qs_oracle as orc
from qspace_gb300 import _capi
from qspace_gb300.linalg import svd_keep
from tests.golden.golden_io import unpack

G = Path(__file__).resolve().parent / "golden"


def _cases():
    z = np.load(G / "svd_golden.npz")
    return z, json.loads(str(z["cases"]))


def _effective(opts):
    nkeep = int(opts.get("Nkeep", -1))
    stol = float(opts["stol"]) if "stol" in opts else (0.0 if nkeep > 0 else 1e-8)
    return nkeep, int(opts.get("Nkmin", 0)), stol


def _blocks(A):
    return [np.linalg.svd(np.asarray(d), compute_uv=False) for d in A["data"]]


@pytest.mark.parametrize("impl", ["oracle", "library"])
def test_svd_truncation_matches_reference(impl):
    z, cases = _cases()
    assert len(cases) == 16
    for c in cases:
        A, Sref = unpack(f"{c['name']}_A", z), unpack(f"{c['name']}_S", z)
        S = _blocks(A)
        assert np.allclose(np.sort(np.concatenate(S))[::-1], z[f"{c['name']}_svd"], rtol=1e-13, atol=1e-14)
        nkeep, nkmin, stol = _effective(c["opts"])
        if impl == "oracle":
            keep, nk, s2t, tot, sfac = orc.svd_keep(S, nkeep, nkmin, stol)
        else:
            keep, nk, s2t, tot, sfac = svd_keep(S, nkeep, nkmin, stol)
        assert nk == c["Nkeep"], c
        assert abs(sfac - c["sfac"]) <= 1e-13 * c["sfac"], c
        assert abs(s2t / tot - c["svd2tr"]) <= 1e-13, c
        got = {tuple(np.asarray(A["Q"][0][i]).ravel()): S[i][keep[i]] * sfac for i in range(len(S)) if keep[i].any()}
        # the reference's S blocks are diagonals stored as (k, 1) vectors
        ref = {tuple(np.asarray(Sref["Q"][0][i]).ravel()): np.sort(np.abs(np.asarray(d).ravel()))[::-1]
               for i, d in enumerate(Sref["data"])}
        assert got.keys() == ref.keys(), c["name"]
        for k in ref:
            assert np.allclose(got[k], ref[k], rtol=1e-13, atol=1e-14), (c["name"], k)
