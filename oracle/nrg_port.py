"""CPU counterpart of the NRG iteration driver -- TEST INFRASTRUCTURE ONLY.

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
        Q0, data = [], []
        for i in range(n):
            k = int(keep[i].sum())
            if k:
                Q0.append(np.asarray(H["Q"][0][i]).ravel())
                data.append(U[i][:, :k])
        Q = np.array(Q0, np.int32)
        AK = {"Q": [Q, Q.copy()], "data": data, "info": {}} if data else {"Q": [], "data": [], "info": {}}
        return labels, E, keep, AK


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
