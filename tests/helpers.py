"""Shared comparison helpers for the parity tests."""
from __future__ import annotations

import numpy as np


def as_dict(X):
    if isinstance(X, dict):
        return X
    return X.to_dict()


def rel_err(C, R) -> float:
    """Relative Frobenius error over all blocks (C vs reference R)."""
    C, R = as_dict(C), as_dict(R)
    num = den = 0.0
    for c, r in zip(C["data"], R["data"]):
        c = np.asarray(c)
        r = np.asarray(r)
        num += float(np.sum(np.abs(c.reshape(r.shape) - r) ** 2))
        den += float(np.sum(np.abs(r) ** 2))
    if den == 0.0:
        return 0.0 if num == 0.0 else float("inf")
    return float(np.sqrt(num / den))


def assert_same_structure(C, R):
    """Block count, labels (bit-exact) and block shapes identical."""
    C, R = as_dict(C), as_dict(R)
    assert len(C["data"]) == len(R["data"]), (len(C["data"]), len(R["data"]))
    if not R["data"]:
        return
    assert len(C["Q"]) == len(R["Q"]), "rank differs"
    for k, (qc, qr) in enumerate(zip(C["Q"], R["Q"])):
        qc = np.asarray(qc).reshape(len(C["data"]), -1)
        qr = np.asarray(qr).reshape(len(R["data"]), -1)
        assert np.array_equal(qc.astype(np.int64), qr.astype(np.int64)), f"labels of leg {k + 1} differ"
    r = len(R["Q"])
    for i, (c, x) in enumerate(zip(C["data"], R["data"])):
        sc = tuple(np.shape(c)) + (1,) * (r - np.ndim(c))
        sx = tuple(np.shape(x)) + (1,) * (r - np.ndim(x))
        assert sc[:max(r, 1)] == sx[:max(r, 1)] or int(np.prod(sc)) == int(np.prod(sx)) == 1, \
            f"block {i} shape {sc} vs {sx}"


def assert_qspace_close(C, R, tol: float):
    assert_same_structure(C, R)
    e = rel_err(C, R)
    assert e <= tol, f"relative error {e:.3e} > {tol:.1e}"
    return e
