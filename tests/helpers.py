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


def svd_bond_legs(r: int, idx, permA=None, permB=None):
    """0-based positions of the new bond in svdQS's U and Vd: Vd gets it
    first, a single split-off leg leaves U in PSI's leg order, a single kept
    leg leaves Vd in it (Source/svdQS.cc:209-229), then permA / permB."""
    I = [int(i) - 1 for i in idx]
    K = r - len(I)
    P = [i for i in range(r) if i not in I] + I
    iP = [int(x) for x in np.argsort(P)]
    n = r - K + 1
    pb = [n - 1] + list(range(n - 1))
    if permB:
        pb = [pb[j - 1] for j in permB]
    pa = [j - 1 for j in permA] if permA else None
    if K + 1 == r:
        pa = [iP[j] for j in pa] if pa else iP
    elif K == 1:
        pb = [iP[j] for j in pb]
    return (pa.index(K) if pa else K), pb.index(r - K)


def _padded(X, i):
    r = len(X["Q"])
    d = np.asarray(X["data"][i])
    return d.reshape((tuple(d.shape) + (1,) * r)[:r] if d.ndim < r else d.shape, order="F")


def svd_factors(U, S, V, bu: int, bv: int):
    """Per block of S: (U rows stacked over U's blocks on that bond label,
    the singular values, Vd columns side by side over Vd's blocks)."""
    U, S, V = as_dict(U), as_dict(S), as_dict(V)
    nU, nS, nV = len(U["data"]), len(S["data"]), len(V["data"])
    qU = np.asarray(U["Q"][bu]).reshape(nU, -1) if nU else None
    qV = np.asarray(V["Q"][bv]).reshape(nV, -1) if nV else None
    out = []
    for j in range(nS):
        s = np.asarray(S["data"][j]).ravel()
        lu = np.asarray(S["Q"][0]).reshape(nS, -1)[j]
        lv = np.asarray(S["Q"][1]).reshape(nS, -1)[j]
        ub = [np.moveaxis(_padded(U, i), bu, -1).reshape(-1, s.size, order="F")
              for i in range(nU) if np.array_equal(qU[i], lu)]
        vb = [np.moveaxis(_padded(V, i), bv, 0).reshape(s.size, -1, order="F")
              for i in range(nV) if np.array_equal(qV[i], lv)]
        out.append((np.vstack(ub), s, np.hstack(vb)))
    return out


def assert_svd_matches(got, refd, idx, opts, tol: float = 1e-11):
    """svdQS outputs against the reference's: labels, block order, shapes and
    itags exactly; the singular values and, per bond sector, U diag(S) Vd
    (free of the singular vectors' phases) within tol; U and Vd isometric."""
    for g, x in zip(got, refd):
        assert_same_structure(g, x)
        assert (as_dict(g)["info"].get("itags") or None) == (as_dict(x)["info"].get("itags") or None)
    r = len(as_dict(got[0])["Q"]) if as_dict(got[0])["data"] else None
    if r is None:
        assert not as_dict(refd[0])["data"]
        return
    rank = len(as_dict(got[0])["Q"]) + len(as_dict(got[2])["Q"]) - 2
    bu, bv = svd_bond_legs(rank, idx, opts.get("permA"), opts.get("permB"))
    for (gu, gs, gv), (xu, xs, xv) in zip(svd_factors(*got, bu, bv), svd_factors(*refd, bu, bv)):
        assert np.allclose(gs, xs, rtol=tol, atol=tol * xs.max())
        smax = xs.max()
        assert np.abs((gu * gs) @ gv - (xu * xs) @ xv).max() <= tol * smax * 10
        assert np.abs(gu.conj().T @ gu - np.eye(gs.size)).max() <= tol * 10
        assert np.abs(gv @ gv.conj().T - np.eye(gs.size)).max() <= tol * 10


def _bond_stack(X, b: int, label, first: bool, nk=None):
    X = as_dict(X)
    n = len(X["data"])
    q = np.asarray(X["Q"][b]).reshape(n, -1)
    parts = []
    for i in range(n):
        if not np.array_equal(q[i], label):
            continue
        d = _padded(X, i)
        k = d.shape[b]
        parts.append(np.moveaxis(d, b, 0).reshape(k, -1, order="F") if first
                     else np.moveaxis(d, b, -1).reshape(-1, k, order="F"))
    return np.hstack(parts) if first else np.vstack(parts)


def assert_ortho_matches(got, refd, b1: int, b2: int, tol: float = 1e-11, iso: int = 1):
    """orthoQS's [A1, A2] against the reference's: labels, block order,
    shapes and itags exactly; per bond label, A1 A2 contracted over the bond
    (free of the singular vectors' phases) within tol, and A<iso> (the U
    factor) isometric.  b1 / b2: the bond's leg in A1 / A2."""
    for g, x in zip(got, refd):
        assert_same_structure(g, x)
        assert (as_dict(g)["info"].get("itags") or None) == (as_dict(x)["info"].get("itags") or None)
    A1 = as_dict(got[0])
    if not A1["data"]:
        return
    n1 = len(A1["data"])
    labels = {tuple(x) for x in np.asarray(A1["Q"][b1]).reshape(n1, -1)}
    for lab in sorted(labels):
        lab = np.array(lab)
        gu, xu = _bond_stack(got[0], b1, lab, False), _bond_stack(refd[0], b1, lab, False)
        gv, xv = _bond_stack(got[1], b2, lab, True), _bond_stack(refd[1], b2, lab, True)
        scale = max(np.abs(xv).max(), 1.0)
        assert np.abs(gu @ gv - xu @ xv).max() <= tol * scale * 10
        W = gu.conj().T @ gu if iso == 1 else gv @ gv.conj().T
        assert np.abs(W - np.eye(W.shape[0])).max() <= tol * 10
