"""Generates the golden fixture of the Wilson-chain NRG iteration from the
REFERENCE itself: qspace_gb300.nrg.step run on the reference's own contractQS,
permuteQS, plusQS and eigQS MEX sources compiled unmodified against the fake
MATLAB runtime (oracle/refbuild.py, oracle/nrg_port.RefBackend).

    python -m oracle.refbuild contractQS permuteQS plusQS eigQS
    python tests/golden/make_nrg_golden.py

Writes tests/golden/nrg_golden.npz: for each run (the spinful U(1)xU(1)
chain with impurity level eps and interaction U, Lambda, z-shift, kept
states, degeneracy window deps) and iteration: the states before and after
the truncation, every level of the iteration as the reference's eigQS
reports it (ascending, averaged over degenerate clusters), and the kept
states per symmetry sector.
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
from oracle.nrg_port import RefBackend  # noqa: E402
from qspace_gb300.nrg import initial_space, step, wilson_hopping  # noqa: E402

RUNS = [
    {"name": "run0", "eps": -0.2, "U": 0.6, "Lambda": 2.5, "z": 0.0, "nkeep": 200, "deps": 1e-8, "iters": 12},
    {"name": "run1", "eps": -0.35, "U": 0.7, "Lambda": 3.0, "z": 0.5, "nkeep": 128, "deps": 1e-6, "iters": 10},
    {"name": "run2", "eps": -0.1, "U": 0.3, "Lambda": 2.0, "z": 0.25, "nkeep": 512, "deps": 1e-8, "iters": 9},
]


def main():
    for name in ("contractQS", "permuteQS", "plusQS", "eigQS"):
        if not ref.available(name):
            sys.exit("build the reference oracle first: python -m oracle.refbuild contractQS permuteQS plusQS eigQS")
    z = {}
    be = RefBackend()
    for r in RUNS:
        K = initial_space(be, r["eps"], r["U"])
        for n in range(r["iters"]):
            K = step(K, be, wilson_hopping(n, r["Lambda"], r["z"]), r["Lambda"], nkeep=r["nkeep"], deps=r["deps"])
            key = f"{r['name']}_{n}"
            z[key + "_E"] = K.Eall
            labs = sorted(K.E)
            z[key + "_labels"] = np.array(labs, np.int32).reshape(len(labs), -1)
            z[key + "_kept"] = np.array([len(K.E[l]) for l in labs], np.int64)
            z[key + "_sizes"] = np.array([K.nkept, K.ntotal], np.int64)
    z["runs"] = np.array(json.dumps(RUNS))
    np.savez_compressed(os.path.join(HERE, "nrg_golden.npz"), **z)
    print("wrote nrg_golden.npz with", len(RUNS), "runs in", HERE)


if __name__ == "__main__":
    main()
