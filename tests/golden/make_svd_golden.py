"""Generates the golden fixtures of svdQS's truncation from the REFERENCE
itself: QSpace's own svdQS MEX source compiled unmodified against the fake
MATLAB runtime (oracle/refbuild.py, oracle/ref.py).

    python -m oracle.refbuild svdQS
    python tests/golden/make_svd_golden.py

Writes tests/golden/svd_golden.npz: seeded block-diagonal rank-2 PSIs (one
block per left label, so that every block is its own SVD), the options
(Nkeep, Nkmin, stol), and the reference's outputs: the singular values in
descending order, the kept count, the discarded weight fraction, the total
weight, the rescale factor sfac and the kept (rescaled) singular values per
block label.
"""
from __future__ import annotations

import ctypes as C
import json
import os
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))
sys.path.insert(0, ROOT)

from oracle import ref  # noqa: E402
from tests.golden.golden_io import pack  # noqa: E402

# (options): Nkeep / Nkmin / stol as given to svdQS (None: not given)
OPTIONS = [
    {"Nkeep": 6}, {"Nkeep": 1}, {"Nkeep": 40}, {"stol": 0.5}, {"stol": 1.5, "Nkmin": 5},
    {"Nkeep": 8, "stol": 1.0}, {}, {"Nkeep": 12, "stol": 3.0, "Nkmin": 2},
]


def psi(seed: int, cplx: bool):
    rng = np.random.default_rng(seed)
    nb = int(rng.integers(3, 7))
    labs = sorted({(int(a), int(b)) for a, b in rng.integers(-3, 4, size=(nb, 2))})
    data = []
    for _ in labs:
        m, n = (int(x) for x in rng.integers(1, 9, 2))
        x = rng.standard_normal((m, n)) * rng.uniform(0.2, 3.0)
        data.append(x + 1j * rng.standard_normal((m, n)) if cplx else x)
    Q = np.array(labs, np.int32)
    return {"Q": [Q, Q.copy()], "data": data, "info": {"itags": ["L", "R*"]}}


def field(lib, S, name):
    a = lib.mxGetField(S, 0, name.encode())
    return ref._np_of(a) if a else None


def main():
    if not ref.available("svdQS"):
        sys.exit("build the reference oracle first: python -m oracle.refbuild svdQS")
    lib = ref._fake()
    z, meta = {}, []
    for c, opts in enumerate(OPTIONS):
        for cplx in (False, True):
            name = f"svd{c}_{int(cplx)}"
            A = psi(100 + 7 * c + int(cplx), cplx)
            args = [ref.to_mx(A), ref._arg([2])]
            for k, v in opts.items():
                args += [ref._mx_string(k), ref._arg(v)]
            U, S, V, info = ref.call("svdQS", args, 4)
            Sq = ref.from_mx(S)
            pack(f"{name}_A", A, z)
            pack(f"{name}_S", Sq, z)
            res = {k: field(lib, info, k) for k in ("svd", "svd2tr", "sv2tot", "sfac", "Nkeep", "Ntot")}
            z[f"{name}_svd"] = np.asarray(res["svd"], float).reshape(-1)
            meta.append({"name": name, "opts": opts, "Nkeep": int(res["Nkeep"].ravel()[0]),
                         "Ntot": int(res["Ntot"].ravel()[0]), "sfac": float(res["sfac"].ravel()[0]),
                         "svd2tr": float(res["svd2tr"].ravel()[0]), "sv2tot": float(res["sv2tot"].ravel()[0])})
            for x in (U, S, V, info) + tuple(args):
                lib.mxDestroyArray(x)
    z["cases"] = np.array(json.dumps(meta))
    np.savez_compressed(os.path.join(HERE, "svd_golden.npz"), **z)
    print("wrote svd_golden.npz with", len(meta), "cases in", HERE)


if __name__ == "__main__":
    main()
