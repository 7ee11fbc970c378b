"""Generates the golden fixtures of eigQS's truncation from the REFERENCE
itself: QSpace's own eigQS MEX source compiled unmodified against the fake
MATLAB runtime (oracle/refbuild.py, oracle/ref.py).

    python -m oracle.refbuild eigQS
    python tests/golden/make_eig_golden.py

Writes tests/golden/eig_golden.npz: seeded block-diagonal real symmetric
rank-2 H (some sectors repeat another's block, so levels are exactly
degenerate across sectors), the options (Nkeep, Etrunc, deps) and the
reference's outputs: the kept count NK, the truncation energy Etrunc and the
kept eigenvalues EK of every sector and all levels Etot (ascending; with
deps > 0 both hold markSet's averaged levels).  (The reference's NK equals the number
of kept states except with Etrunc > 0 and deps = 0, where it stays
min(Nkeep, N); EK always holds the kept states.)
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

OPTIONS = [
    {"Nkeep": 10}, {"Nkeep": 25}, {"Nkeep": 25, "deps": 1e-8}, {"Nkeep": 40, "deps": 1e-3},
    {"Etrunc": 1.5}, {"Nkeep": 30, "Etrunc": 2.0}, {"Nkeep": 500}, {"Nkeep": 17, "deps": 1e-6},
    {"Etrunc": 0.8, "deps": 1e-6}, {"Nkeep": 60, "Etrunc": 2.5, "deps": 1e-8},
    # near-degenerate sectors (copies perturbed by ~1e-10): markSet averages
    # the clusters and eigQS reports the averaged levels
    {"Nkeep": 25, "deps": 1e-8, "near": 1e-10}, {"Nkeep": 40, "deps": 1e-6, "near": 1e-9},
    {"Nkeep": 500, "deps": 1e-6, "near": 1e-10}, {"Etrunc": 1.0, "deps": 1e-7, "near": 3e-10},
]


def hamiltonian(seed: int, near: float = 0.0):
    rng = np.random.default_rng(seed)
    labs = sorted({(int(a), int(b)) for a, b in rng.integers(-3, 4, size=(int(rng.integers(7, 11)), 2))})
    data = []
    for i, _ in enumerate(labs):
        if i and rng.uniform() < 0.35:
            x = data[int(rng.integers(0, i))].copy()     # degenerate with an earlier sector
            if near:
                y = rng.standard_normal(x.shape)
                x = x + near * (y + y.T) / 2               # ... up to ~near
            data.append(x)
            continue
        n = int(rng.integers(3, 21))
        x = rng.standard_normal((n, n))
        data.append((x + x.T) / 2)
    Q = np.array(labs, np.int32)
    return {"Q": [Q, Q.copy()], "data": data, "info": {}}


def main():
    if not ref.available("eigQS"):
        sys.exit("build the reference oracle first: python -m oracle.refbuild eigQS")
    lib = ref._fake()
    z, meta = {}, []
    for c, opts in enumerate(OPTIONS):
        name = f"eig{c}"
        H = hamiltonian(200 + c, opts.get("near", 0.0))
        args = [ref.to_mx(H)]
        for k, v in opts.items():
            if k != "near":
                args += [ref._mx_string(k), ref._arg(v)]
        Etot, I = ref.call("eigQS", args, 2)
        EK = ref.from_mx(lib.mxGetField(I, 0, b"EK"))
        nk = int(ref._np_of(lib.mxGetField(I, 0, b"NK")).ravel()[0])
        et = float(ref._np_of(lib.mxGetField(I, 0, b"Etrunc")).ravel()[0])
        pack(f"{name}_H", H, z)
        pack(f"{name}_EK", EK, z)
        z[f"{name}_Etot"] = ref._np_of(Etot).ravel().copy()
        meta.append({"name": name, "opts": opts, "NK": nk, "Etrunc": et})
        for x in (Etot, I) + tuple(args):
            lib.mxDestroyArray(x)
    z["cases"] = np.array(json.dumps(meta))
    np.savez_compressed(os.path.join(HERE, "eig_golden.npz"), **z)
    print("wrote eig_golden.npz with", len(meta), "cases in", HERE)


if __name__ == "__main__":
    main()
