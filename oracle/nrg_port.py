"""CPU counterpart of the NRG iteration driver -- TEST INFRASTRUCTURE ONLY.

``RefBackend`` runs the same step on the reference's own compiled MEX
functions (the fixture generator tests/golden/make_nrg_golden.py uses it).
``OracleBackend`` runs ``qspace_gb300.nrg.step`` on host QSpace dicts with the
oracle's numpy restatements (contractQS, permuteQS, plusQS, eigQS: numpy
``eigh`` per block + the markSet restatement), so the same iteration is the
checker of the device run and the timed CPU baseline.  ``dense_chain`` builds
the same Wilson chain as one dense matrix (Kronecker products with the
Jordan-Wigner sign) for exact diagonalisation of short chains.  Only
``tests/`` and ``bench.py``'s CPU legs use this module.
"""
from __future__ import annotations

import math

import numpy as np

from oracle import qs_oracle as orc


class OracleBackend:
    def put(self, A):
        return A.to_dict()

    def contract(self, A, ia, B, ib):
        return orc.contract(A, ia, B, ib)

    def permute(self, A, perm, conj=False):
        return orc.permute(A, perm, conj)

    def plus(self, A, B, f):
        return orc.plus(A, B, f)

    def eig(self, H, nkeep, deps=0.0):
        n = len(H["data"])
        labels, E, U = [], [], []
        for i in range(n):
            labels.append(tuple(int(x) for x in np.asarray(H["Q"][0][i]).ravel()))
            e, u = np.linalg.eigh(np.asarray(H["data"][i]).reshape(orc.block_dims(H, i), order="F"))
            E.append(e)
            U.append(u)
        keep, _ = orc.mark_keep(E, nkeep, 0.0, deps)
        keep = [np.asarray(k, bool) for k in keep]
        E = orc.average_levels(E, deps)       # as eigQS reports them (markSet writes them back)
        Q0, data = [], []
        for i in range(n):
            k = int(keep[i].sum())
            if k:
                Q0.append(np.asarray(H["Q"][0][i]).ravel())
                data.append(U[i][:, :k])
        Q = np.array(Q0, np.int32)
        AK = {"Q": [Q, Q.copy()], "data": data, "info": {}} if data else {"Q": [], "data": [], "info": {}}
        return labels, E, keep, AK


class RefBackend:
    """The iteration on the REFERENCE's own MEX functions compiled here
    (oracle/refbuild.py: contractQS, permuteQS, plusQS, eigQS behind the fake
    MATLAB runtime): the chain that pins the device iteration.  eigQS's
    outputs are taken as the reference reports them (levels after markSet's
    degeneracy averaging when deps > 0).

    The reference's QSpace routines expect an itag per leg (with none,
    permuteQS stops on the empty tag list and contractQS crashes), while the
    iteration's tensors carry none: every call but eigQS (which accepts an
    untagged operator) gets empty tags, which match
    any leg (Source/wbindex.cc:989-1005).  Contracted legs then point the same
    way and the reference toggles the first operand's conjugation, which
    leaves the real tensors of this chain unchanged; the tags are dropped
    from the results again."""

    @staticmethod
    def _tagged(A):
        if (A.get("info") or {}).get("itags"):
            return A
        return dict(A, info={"itags": [""] * len(A["Q"])})

    @staticmethod
    def _plain(R):
        R["info"] = {}
        return R

    def put(self, A):
        return A.to_dict()

    def contract(self, A, ia, B, ib):
        from oracle import ref
        return self._plain(ref.contractQS(self._tagged(A), ia, self._tagged(B), ib))

    def permute(self, A, perm, conj=False):
        from oracle import ref
        return self._plain(ref.permuteQS(self._tagged(A), perm, conj))

    def plus(self, A, B, f):
        from oracle import ref
        return self._plain(ref.plusQS(self._tagged(A), self._tagged(B), f))

    def eig(self, H, nkeep, deps=0.0):
        from oracle import ref
        opts = {"Nkeep": int(nkeep)}
        if deps > 0:
            opts["deps"] = float(deps)
        _, I = ref.eigQS(dict(H, info={}), **opts)     # eigQS takes no tags or operator tags
        lab = lambda X, i: tuple(int(x) for x in np.asarray(X["Q"][0][i]).ravel())
        ek = {lab(I["EK"], i): np.asarray(d, float).ravel() for i, d in enumerate(I["EK"]["data"])}
        ed = {lab(I["ED"], i): np.asarray(d, float).ravel() for i, d in enumerate(I["ED"]["data"])}
        labels, E, keep = [], [], []
        for i in range(len(H["data"])):
            k = lab(H, i)
            a, b = ek.get(k, np.zeros(0)), ed.get(k, np.zeros(0))
            labels.append(k)
            E.append(np.concatenate([a, b]))
            keep.append(np.arange(len(a) + len(b)) < len(a))
        return labels, E, keep, self._plain(I["AK"])


def dense_chain(L: int, eps: float, U: float, ts, Lam: float) -> np.ndarray:
    """All eigenvalues of H_{L-1} of the recursion H_0 = eps n + U n_up n_dn,
    H_{N+1} = sqrt(Lam) H_N + t_N sum_s (f_{N,s}^+ f_{N+1,s} + h.c.), built as
    dense matrices (site basis |0>, |up>, |dn>, |updn>)."""
    cu = np.zeros((4, 4)); cu[0, 1] = 1; cu[2, 3] = 1
    cd = np.zeros((4, 4)); cd[0, 2] = 1; cd[1, 3] = -1
    Z = np.diag([1.0, -1.0, -1.0, 1.0])
    H = eps * np.diag([0.0, 1.0, 1.0, 2.0]) + U * np.diag([0.0, 0.0, 0.0, 1.0])
    F = {"up": cu, "dn": cd}
    Zt = Z
    for N in range(L - 1):
        H = math.sqrt(Lam) * np.kron(H, np.eye(4))
        for s, c in (("up", cu), ("dn", cd)):
            hop = np.kron(F[s].T @ Zt, c)
            H = H + ts[N] * (hop + hop.T)
        F = {"up": np.kron(Zt, cu), "dn": np.kron(Zt, cd)}
        Zt = np.kron(Zt, Z)
    return np.linalg.eigvalsh(H)
