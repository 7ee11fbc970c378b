"""Generates the golden fixtures of the QSpace-level svdQS and orthoQS from
the REFERENCE itself: QSpace's own svdQS and orthoQS MEX sources compiled
unmodified against the fake MATLAB runtime (oracle/refbuild.py,
oracle/ref.py).

    python -m oracle.refbuild svdQS orthoQS
    python tests/golden/make_svdqs_golden.py

Writes tests/golden/svdqs_golden.npz: seeded abelian PSIs of rank 2 to 4
(labels conserved at every block, one or two label components, real and
complex, legs pointing in and out), the split-off legs and the options, and
the reference's [U, S, Vd, info]: labels, block order, block shapes, itags,
data, and from info the kept count, the rescale factor sfac, the discarded
weight svd2tr, the flag and all singular values; for orthoQS (usage #1
without lrdir and #2 with it) the same for [A1, A2, info].  Cases the
reference rejects are stored with their error flag only.
"""
from __future__ import annotations

import json
import os
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))
sys.path.insert(0, ROOT)

from oracle import ref  # noqa: E402
from tests.golden.golden_io import pack  # noqa: E402

# (itags, split-off legs, options, complex, label components)
CASES = [
    (["a", "b*"], [2], {}, False, 1),
    (["a", "b*"], [1], {"Nkeep": 4}, True, 1),
    (["a", "b"], [2], {}, False, 1),
    (["a", "b"], [1], {"stol": 0.5}, True, 2),
    (["a*", "b*"], [2], {"Nkeep": 5, "Nkmin": 2, "stol": 1.0}, False, 1),
    (["a*", "b"], [1], {"itag": "X"}, False, 2),
    (["L", "s", "R*"], [3], {}, False, 1),
    (["L", "s", "R*"], [3], {"Nkeep": 6}, True, 2),
    (["L", "s", "R*"], [2, 3], {"stol": 0.3}, False, 1),
    (["L", "s", "R*"], [1, 2], {"itag": "K"}, True, 1),
    (["L", "s", "R*"], [3, 2], {"Nkeep": 5}, False, 2),
    (["L", "s", "R*"], [1], {}, False, 1),                       # rejected: mixed group
    (["a", "b", "c"], [3], {}, False, 1),
    (["a", "b", "c"], [1], {"Nkeep": 7}, True, 1),
    (["a", "b", "c"], [2], {"stol": 0.8, "Nkmin": 3}, False, 2),
    (["a", "b", "c"], [1, 2], {}, True, 2),
    (["a*", "b*", "c*"], [2, 3], {"Nkeep": 3}, False, 1),
    (["a", "b", "c"], [3], {"permA": [3, 1, 2]}, False, 1),
    (["L", "s", "R*"], [2, 3], {"permB": [2, 3, 1]}, True, 1),
    (["L", "s", "R*"], [3], {"permA": [2, 1, 3], "permB": [2, 1]}, False, 2),
    (["a", "b", "c*", "d*"], [3, 4], {}, False, 1),
    (["a", "b", "c*", "d*"], [3, 4], {"Nkeep": 8}, True, 2),
    (["L", "s1", "s2", "R*"], [4], {"stol": 0.2}, False, 1),
    (["L", "s1", "s2", "R*"], [2, 3, 4], {"Nkeep": 6}, True, 1),
    (["a", "b", "c", "d"], [4], {"itag": "Y*"}, False, 1),
    (["a", "b", "c", "d"], [1], {}, True, 2),
    (["a", "b", "c*", "d"], [3, 4], {}, False, 1),               # rejected: mixed right group
    (["L", "s", "R*"], [3], {"Nkeep": 0}, False, 1),             # nothing kept: empty outputs
]

# orthoQS: (itags, legs, lrdir or None, options, complex, label components)
ORTHO_CASES = [
    (["a", "b*"], [1], None, {}, False, 1),
    (["L", "s", "R*"], [3], None, {"Nkeep": 5}, True, 1),
    (["L", "s", "R*"], [1], None, {"stol": 0.4}, False, 2),
    (["a", "b", "c"], [2], None, {}, True, 1),
    (["L", "s", "R*"], [1, 2], ">>", {}, False, 1),
    (["L", "s", "R*"], [3], "<<", {"Nkeep": 6}, True, 1),
    (["L", "s", "R*"], [1], ">>", {"itag": "K"}, False, 2),
    (["L", "s", "R*"], [2, 3], "<<", {}, False, 1),
    (["a", "b", "c"], [1, 2], "LR", {"permA": [2, 1, 3]}, False, 1),
    (["a", "b", "c"], [3], "RL", {"permB": [2, 1]}, True, 2),
    (["a", "b*"], [2], "+", {"Nkeep": 3}, False, 1),
    (["a", "b"], [1], "-", {"stol": 0.5, "Nkmin": 2}, True, 1),
    (["a", "b", "c*", "d*"], [1, 2], ">>", {}, False, 1),
    (["a", "b", "c*", "d*"], [3, 4], "<<", {"Nkeep": 7, "itag": "Y*"}, True, 1),
    (["L", "s1", "s2", "R"], [1, 2], "LR", {"permB": [3, 1, 2]}, False, 2),
    (["a", "b", "c*", "d"], [3, 4], "LR", {}, False, 1),            # rejected: mixed right group
    (["L", "s", "R*"], [1, 2], ">>", {"Nkeep": 0}, False, 1),       # nothing kept
]


def psi(seed: int, tags: list, cplx: bool, qdim: int, nb: int = 7) -> dict:
    """Random abelian PSI: labels in [-2, 2], the last leg's label fixed by
    conservation (ingoing labels minus outgoing ones sum to zero), sector
    dimensions 1..3 fixed per (leg, label)."""
    rng = np.random.default_rng(seed)
    r = len(tags)
    sgn = np.array([-1 if t.endswith("*") else 1 for t in tags])
    recs = set()
    for _ in range(500):
        if len(recs) == nb:
            break
        q = rng.integers(-2, 3, size=(r - 1, qdim))
        last = -sgn[-1] * (sgn[:-1, None] * q).sum(axis=0)
        recs.add(tuple(map(tuple, np.vstack([q, last[None]]))))
    recs = sorted(recs)
    sec, data = {}, []
    for rec in recs:
        shp = [sec.setdefault((k, rec[k]), int(rng.integers(1, 4))) for k in range(r)]
        x = rng.standard_normal(shp)
        data.append(x + 1j * rng.standard_normal(shp) if cplx else x)
    Q = [np.array([rec[k] for rec in recs], np.int32) for k in range(r)]
    return {"Q": Q, "data": data, "info": {"itags": list(tags)}}


def field(lib, S, name):
    a = lib.mxGetField(S, 0, name.encode())
    return ref._np_of(a) if a else None


def main():
    if not (ref.available("svdQS") and ref.available("orthoQS")):
        sys.exit("build the reference oracle first: python -m oracle.refbuild svdQS orthoQS")
    lib = ref._fake()
    z, meta = {}, []
    for c, (tags, idx, opts, cplx, qdim) in enumerate(CASES):
        name = f"svdqs{c}"
        A = psi(300 + c, tags, cplx, qdim)
        args = [ref.to_mx(A), ref._arg(idx)]
        for k, v in opts.items():
            args += [ref._mx_string(k), ref._arg(v)]
        pack(f"{name}_A", A, z)
        m = {"name": name, "idx": idx, "opts": opts}
        try:
            U, S, V, info = ref.call("svdQS", args, 4)
        except ref.RefError:
            m["error"] = True
            meta.append(m)
            continue
        for tag, X in (("U", U), ("S", S), ("V", V)):
            pack(f"{name}_{tag}", ref.from_mx(X), z)
        z[f"{name}_svd"] = np.asarray(field(lib, info, "svd"), float).reshape(-1)
        for k in ("Nkeep", "Ntot", "flag"):
            m[k] = int(field(lib, info, k).ravel()[0])
        for k in ("sfac", "svd2tr", "sv2tot"):
            m[k] = float(field(lib, info, k).ravel()[0])
        meta.append(m)
        for x in (U, S, V, info) + tuple(args):
            lib.mxDestroyArray(x)
    ometa = []
    for c, (tags, idx, lrdir, opts, cplx, qdim) in enumerate(ORTHO_CASES):
        name = f"ortho{c}"
        A = psi(600 + c, tags, cplx, qdim)
        args = [ref.to_mx(A), ref._arg(idx)] + ([ref._mx_string(lrdir)] if lrdir else [])
        for k, v in opts.items():
            args += [ref._mx_string(k), ref._arg(v)]
        pack(f"{name}_A", A, z)
        m = {"name": name, "idx": idx, "lrdir": lrdir, "opts": opts}
        try:
            A1, A2, info = ref.call("orthoQS", args, 3)
        except ref.RefError:
            m["error"] = True
            ometa.append(m)
            continue
        pack(f"{name}_A1", ref.from_mx(A1), z)
        pack(f"{name}_A2", ref.from_mx(A2), z)
        for k in ("Nkeep", "flag"):
            m[k] = int(field(lib, info, k).ravel()[0])
        m["sfac"] = float(field(lib, info, "sfac").ravel()[0])
        ometa.append(m)
        for x in (A1, A2, info) + tuple(args):
            lib.mxDestroyArray(x)
    z["cases"] = np.array(json.dumps(meta))
    z["ortho_cases"] = np.array(json.dumps(ometa))
    np.savez_compressed(os.path.join(HERE, "svdqs_golden.npz"), **z)
    print("wrote svdqs_golden.npz with", len(meta), "svdQS and", len(ometa), "orthoQS cases,",
          sum("error" in m for m in meta + ometa), "rejected")


if __name__ == "__main__":
    main()
