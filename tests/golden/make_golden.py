"""Generates the golden fixtures of the contraction path from the REFERENCE
itself: QSpace's own contractQS / permuteQS MEX sources compiled unmodified
against the fake MATLAB runtime (oracle/refbuild.py, oracle/ref.py).

    python -m oracle.refbuild contractQS permuteQS
    python tests/golden/make_golden.py

Writes tests/golden/contract_golden.npz, permute_golden.npz and
cell_golden.npz (itag cell contractions): inputs, index/perm arguments, and
the reference outputs (labels, block order, itags, data).
The inputs are seeded synthetic tensors (qspace_gb300.workloads); the
reference was built with QS_SKIP_MPFR (abelian cases need no CG data).
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
from qspace_gb300 import QSpace  # noqa: E402
from qspace_gb300.workloads import mps_site_tensor, random_abelian, random_leg  # noqa: E402
from tests.golden.golden_io import pack  # noqa: E402

# (A legs, B legs (indices into a shared leg table), ia, ib, perm)
CASES = [
    ((0, 1, 2), (2, 3), "3", "1", None),
    ((0, 1, 2), (2, 1, 3), "2,3", "2,1", None),
    ((0, 1, 2), (1, 3, 0), "1,2", "3,1", "2,1"),
    ((0, 1, 2), (1, 3, 0), "2,1", "1,3", None),
    ((0, 1, 2), (2, 0, 3), "3,1", "1,2", "2,1"),
    ((0, 1, 2, 3), (3, 1, 4), "4,2", "1,2", "3,2,1"),
    ((0, 1), (1, 0), "1,2", "2,1", None),
    ((0, 1, 2), (0, 1, 2), "123", "123", None),
    ((0, 1, 2), (3, 1), "2", "2", "3,2,1"),
]


def contract_cases():
    out = []
    for seed in (1, 2):
        A = mps_site_tensor(seed).to_dict()
        out.append((f"rdm_seed{seed}", A, "12*", A, "12", None))
    for c, (la, lb, ia, ib, perm) in enumerate(CASES):
        for cx in ((False, False), (True, True), (True, False)):
            rng = np.random.default_rng(1000 + 10 * c + 3 * cx[0] + cx[1])
            table = [random_leg(rng, nsec=int(rng.integers(2, 5)), dmax=5, qdim=2) for _ in range(5)]
            # contracted legs carry the same name with opposite directions
            A = random_abelian(rng, [table[i] for i in la], complex_data=cx[0],
                               itags=[f"t{i}" for i in la]).to_dict()
            B = random_abelian(rng, [table[i] for i in lb], complex_data=cx[1],
                               itags=[f"t{i}*" for i in lb]).to_dict()
            conj = "*" if cx[0] else ""
            out.append((f"case{c}_{int(cx[0])}{int(cx[1])}", A, ia + conj, B, ib, perm))
    # zero blocks: dropped for rank 3, kept for a hermitian rank-2 result
    Q1 = np.array([[0], [1]], np.int32)
    A = QSpace([Q1, np.array([[0], [0]], np.int32), np.array([[3], [4]], np.int32)],
               [np.ones((2, 1, 3)), np.zeros((2, 1, 3))], {"itags": ["a", "b", "c"]}).to_dict()
    B = QSpace([Q1, np.array([[7], [7]], np.int32)], [np.ones((2, 2)), np.ones((2, 2))],
               {"itags": ["a*", "d"]}).to_dict()
    out.append(("zero_rank3", A, "1", B, "1", None))
    H = QSpace([Q1, Q1.copy()], [np.eye(2), np.zeros((3, 3))], {"itags": ["x", "x*"]}).to_dict()
    out.append(("zero_rank2_herm", H, "2", H, "1", None))
    # numeric (1-based) index vectors
    rng = np.random.default_rng(77)
    t = [random_leg(rng, nsec=3, dmax=4, qdim=1) for _ in range(4)]
    A = random_abelian(rng, [t[0], t[1], t[2]], itags=["p", "q", "r"]).to_dict()
    B = random_abelian(rng, [t[2], t[3]], itags=["r*", "s"]).to_dict()
    out.append(("numeric_idx", A, [3], B, [1], [2, 1, 3]))
    # same-direction itags without conj flags: the reference conjugates A
    A = random_abelian(rng, [t[0], t[1]], complex_data=True, itags=["u", "v"]).to_dict()
    B = random_abelian(rng, [t[1], t[3]], complex_data=True, itags=["v", "w"]).to_dict()
    out.append(("autoconj", A, "2", B, "1", None))
    return out


def cell_cases():
    """Cell (itag) contractions: [(name, items, perm)], items QSpace dicts or '*'."""
    out = []
    for cx in (False, True):
        rng = np.random.default_rng(4242 + cx)
        t = [random_leg(rng, nsec=3, dmax=4, qdim=2) for _ in range(5)]
        A = random_abelian(rng, [t[0], t[1], t[2]], complex_data=cx, itags=["a", "b", "c"]).to_dict()
        B = random_abelian(rng, [t[2], t[3]], complex_data=cx, itags=["c*", "d"]).to_dict()
        C = random_abelian(rng, [t[3], t[4]], complex_data=cx, itags=["d*", "e"]).to_dict()
        s = f"{'z' if cx else 'r'}"
        out += [(f"pair_{s}", [A, B], None), (f"pair_perm_{s}", [A, B], [3, 1, 2]),
                (f"chain3_{s}", [A, B, C], None), (f"chain3_perm_{s}", [A, B, C], [2, 1]),
                (f"conjA_{s}", [A, "*", B], None), (f"conjlast_{s}", [B, C, "*"], None),
                (f"norm_{s}", [A, "*", A], None)]
    M = mps_site_tensor(3, D=128, complex_data=True).to_dict()
    out.append(("mps_rdm", [M, "*", M], None))
    return out


def main():
    if not ref.available("contractQS") or not ref.available("permuteQS"):
        sys.exit("build the reference oracle first: python -m oracle.refbuild contractQS permuteQS")
    z, meta = {}, []
    for name, A, ia, B, ib, perm in contract_cases():
        C = ref.contractQS(A, ia, B, ib, perm)
        pack(f"{name}_A", A, z)
        pack(f"{name}_B", B, z)
        pack(f"{name}_C", C, z)
        meta.append({"name": name, "ia": ia, "ib": ib, "perm": perm})
    z["cases"] = np.array(json.dumps(meta))
    np.savez_compressed(os.path.join(HERE, "contract_golden.npz"), **z)

    z, meta = {}, []
    rng = np.random.default_rng(5)
    for c, cx in enumerate((False, True)):
        legs = [random_leg(rng, nsec=3, dmax=4, qdim=2) for _ in range(3)]
        A = random_abelian(rng, legs, complex_data=cx, itags=["a", "b*", "c"]).to_dict()
        for perm in ([3, 1, 2], [2, 1, 3]):
            for conj in (False, True):
                name = f"perm{c}_{''.join(map(str, perm))}_{int(conj)}"
                Bp = ref.permuteQS(A, perm, conj)
                pack(f"{name}_A", A, z)
                pack(f"{name}_B", Bp, z)
                meta.append({"name": name, "perm": perm, "conj": conj})
    z["cases"] = np.array(json.dumps(meta))
    np.savez_compressed(os.path.join(HERE, "permute_golden.npz"), **z)

    z, meta = {}, []
    for name, items, perm in cell_cases():
        R = ref.contractQS_cell(items, perm)
        spec = []
        for k, x in enumerate(items):
            if isinstance(x, str):
                spec.append(x)
            else:
                pack(f"{name}_X{k}", x, z)
                spec.append(f"X{k}")
        pack(f"{name}_C", R, z)
        meta.append({"name": name, "items": spec, "perm": perm})
    z["cases"] = np.array(json.dumps(meta))
    np.savez_compressed(os.path.join(HERE, "cell_golden.npz"), **z)
    print("wrote contract_golden.npz, permute_golden.npz, cell_golden.npz in", HERE)


if __name__ == "__main__":
    main()
