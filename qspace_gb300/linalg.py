"""Block eigendecomposition / SVD / Gram-Schmidt through the C-ABI.

* ``eigQS(H, Nkeep=, Etrunc=, deps=)`` mirrors the abelian use of the MEX
  ``eigQS`` (Source/eigQS.cc:27-122 -> QSpace::EigenSymmetric,
  Source/QSpace.cc:4673-4939): every symmetry block of a block-diagonal
  rank-2 QSpace is diagonalised on the GPU in FP64, the global truncation
  (markSet) keeps the Nkeep lowest levels, and the kept / discarded
  eigenvectors come back as QSpaces AK / AD with eigenvalues EK / ED.
* ``svdQS(PSI, idx, ...)`` / ``orthoQS(PSI, idx [, lrdir], ...)`` mirror the
  abelian use of the MEX ``svdQS`` / ``orthoQS`` (Source/svdQS.cc:170-234,
  Source/orthoQS.cc:156-310 -> SVD_Data::blockSVD / dmrgTruncate,
  Source/mpsortho.cc:546-905): the blocks of each conserved label sum form
  one matrix, all of them are decomposed on the GPU in one call, truncated
  together, and U / S / Vd (A1 / A2) come back with the reference's labels,
  block order and itags.
* ``eig_blocks``, ``svd_blocks``, ``gs_reortho``: the raw block operations on
  device buffers (torch tensors used as plain device memory).
"""
from __future__ import annotations

import ctypes as C

import numpy as np

from . import _capi
from ._capi import check
from .qspace import Context, QSpace, default_context

c_i64 = _capi.c_int64_p


def _ptr(a: np.ndarray):
    return a.ctypes.data_as(c_i64)


def eig_blocks(blocks: list, ctx: Context | None = None):
    """Eigen-decomposition of a list of Hermitian matrices on the GPU.
    Returns (list of ascending eigenvalue arrays, list of eigenvector
    matrices)."""
    import torch
    ctx = ctx or default_context()
    cplx = any(np.iscomplexobj(b) for b in blocks)
    dt = np.complex128 if cplx else np.float64
    n = np.array([b.shape[0] for b in blocks], np.int64)
    sizes = n * n
    offs = np.concatenate([[0], np.cumsum(sizes)[:-1]]).astype(np.int64)
    eoffs = np.concatenate([[0], np.cumsum(n)[:-1]]).astype(np.int64)
    H = np.concatenate([np.asarray(b, dt).reshape(-1, order="F") for b in blocks]) if blocks else np.zeros(0, dt)
    dev = torch.device("cuda", ctx.device)
    dH = torch.from_numpy(H.view(np.float64)).to(dev)
    dU = torch.empty_like(dH)
    dE = torch.empty(max(int(n.sum()), 1), dtype=torch.float64, device=dev)
    torch.cuda.synchronize(dev)
    check(ctx.lib.qs_eig_blocks(ctx.h, len(blocks), _ptr(n), _ptr(offs), _ptr(eoffs), C.c_void_p(dH.data_ptr()),
                                C.c_void_p(dE.data_ptr()), C.c_void_p(dU.data_ptr()), 1 if cplx else 0))
    ctx.sync()
    E = dE.cpu().numpy()
    U = dU.cpu().numpy()
    if cplx:
        U = U.view(np.complex128)
    Es = [E[eoffs[i]:eoffs[i] + n[i]].copy() for i in range(len(blocks))]
    Us = [U[offs[i]:offs[i] + sizes[i]].reshape((n[i], n[i]), order="F").copy() for i in range(len(blocks))]
    return Es, Us


def mark_keep(E_blocks: list, nkeep: int = -1, etrunc: float = 0.0, deps: float = 0.0):
    """Global truncation (markSet) on the host through the C-ABI."""
    lib = _capi.load()
    n = np.array([len(e) for e in E_blocks], np.int64)
    E = np.concatenate([np.asarray(e, np.float64) for e in E_blocks]) if E_blocks else np.zeros(0)
    keep = np.zeros(max(len(E), 1), np.uint8)
    nk, et = C.c_int64(), C.c_double()
    check(lib.qs_mark_keep(len(n), _ptr(n), E.ctypes.data_as(_capi.c_double_p), None, int(nkeep), float(etrunc),
                           float(deps), keep.ctypes.data_as(C.POINTER(C.c_uint8)), C.byref(nk), C.byref(et)))
    offs = np.concatenate([[0], np.cumsum(n)[:-1]]).astype(np.int64)
    return [keep[o:o + k].astype(bool) for o, k in zip(offs, n)], nk.value, et.value


def average_levels(E_blocks: list, deps: float) -> list:
    """markSet's degeneracy averaging (qs_average_levels): clusters of levels
    closer than deps times the spectral width replaced by their mean, per
    block in the input order (what eigQS reports when deps > 0)."""
    lib = _capi.load()
    n = np.array([len(e) for e in E_blocks], np.int64)
    E = np.concatenate([np.asarray(e, np.float64) for e in E_blocks]) if E_blocks else np.zeros(0)
    out = np.zeros(max(len(E), 1), np.float64)
    check(lib.qs_average_levels(len(n), _ptr(n), E.ctypes.data_as(_capi.c_double_p), float(deps),
                                out.ctypes.data_as(_capi.c_double_p)))
    offs = np.concatenate([[0], np.cumsum(n)[:-1]]).astype(np.int64)
    return [out[o:o + k].copy() for o, k in zip(offs, n)]


def mark_keep_dev(E_blocks: list, nkeep: int = -1, etrunc: float = 0.0, deps: float = 0.0,
                  ctx: Context | None = None):
    """The same truncation with the eigenvalues on the device
    (qs_mark_keep_dev): the values are uploaded, the flags come back."""
    import torch
    ctx = ctx or default_context()
    n = np.array([len(e) for e in E_blocks], np.int64)
    E = np.concatenate([np.asarray(e, np.float64) for e in E_blocks]) if E_blocks else np.zeros(0)
    dev = torch.device("cuda", ctx.device)
    dE = torch.from_numpy(E.copy()).to(dev)
    dk = torch.zeros(max(len(E), 1), dtype=torch.uint8, device=dev)
    torch.cuda.synchronize(dev)
    nk, et = C.c_int64(), C.c_double()
    check(ctx.lib.qs_mark_keep_dev(ctx.h, len(n), _ptr(n), C.c_void_p(dE.data_ptr()), int(nkeep), float(etrunc),
                                   float(deps), C.c_void_p(dk.data_ptr()), C.byref(nk), C.byref(et)))
    ctx.sync()
    keep = dk.cpu().numpy()
    offs = np.concatenate([[0], np.cumsum(n)[:-1]]).astype(np.int64)
    return [keep[o:o + k].astype(bool) for o, k in zip(offs, n)], nk.value, et.value


def eigQS(H: QSpace, Nkeep: int = -1, Etrunc: float = 0.0, deps: float = 0.0, ctx: Context | None = None):
    """Block eigendecomposition + truncation of a block-diagonal rank-2
    abelian QSpace.  Returns (Etot, I) with Etot the ascending eigenvalues of
    all blocks and I = {'AK','AD','EK','ED','NK'} as in eigQS (with deps > 0
    the levels after markSet's degeneracy averaging, as the reference
    reports them)."""
    if H.rank != 2:
        raise ValueError("eigQS: rank-2 QSpace required")
    for i in range(H.nblk):
        if not np.array_equal(H.Q[0][i], H.Q[1][i]):
            raise ValueError("eigQS: block-diagonal (symmetric) QSpace required")
    blocks = [np.asarray(d).reshape(H.block_dims(i)) for i, d in enumerate(H.data)]
    Es, Us = eig_blocks(blocks, ctx)
    keep, nk, _ = mark_keep(Es, Nkeep, Etrunc, deps)
    if deps > 0:          # markSet writes the averaged levels back (reported by eigQS)
        Es = average_levels(Es, deps)
    parts = {}
    for tag, sel in (("K", True), ("D", False)):
        Q0, Q1, data, EQ, Ed = [], [], [], [], []
        for i, (e, u, k) in enumerate(zip(Es, Us, keep)):
            idx = np.flatnonzero(k == sel)
            if idx.size == 0:
                continue
            Q0.append(H.Q[0][i])
            Q1.append(H.Q[1][i])
            data.append(u[:, idx])
            Ed.append(np.diag(e[idx]))
        if data:
            parts["A" + tag] = QSpace([np.asarray(Q0), np.asarray(Q1)], data, dict(H.info))
            parts["E" + tag] = QSpace([np.asarray(Q0), np.asarray(Q1)], Ed, {})
        else:
            parts["A" + tag] = QSpace([], [], {})
            parts["E" + tag] = QSpace([], [], {})
    parts["NK"] = nk
    Etot = np.sort(np.concatenate(Es)) if Es else np.zeros(0)
    return Etot, parts


def svd_keep(S_blocks: list, nkeep: int = -1, nkmin: int = 0, stol: float = 0.0):
    """The truncation of svdQS on the host (qs_svd_keep): per-block keep
    flags, kept count, discarded and total weight, and the rescale factor
    sfac of the kept singular values."""
    lib = _capi.load()
    k = np.array([len(s) for s in S_blocks], np.int64)
    S = np.concatenate([np.asarray(s, np.float64) for s in S_blocks]) if S_blocks else np.zeros(0)
    keep = np.zeros(max(len(S), 1), np.uint8)
    nk, s2t, tot, sfac = C.c_int64(), C.c_double(), C.c_double(), C.c_double()
    check(lib.qs_svd_keep(len(k), _ptr(k), S.ctypes.data_as(_capi.c_double_p), int(nkeep), int(nkmin), float(stol),
                          keep.ctypes.data_as(C.POINTER(C.c_uint8)), C.byref(nk), C.byref(s2t), C.byref(tot),
                          C.byref(sfac)))
    offs = np.concatenate([[0], np.cumsum(k)]).astype(np.int64)
    return ([keep[offs[i]:offs[i + 1]].astype(bool) for i in range(len(k))], nk.value, s2t.value, tot.value,
            sfac.value)


def svd_blocks(blocks: list, ctx: Context | None = None, max_sweeps: int = 0, tol: float = 0.0):
    """Thin SVD of real or complex blocks on the GPU (qs_svd_blocks_ex):
    returns lists U, S, Vt with A = U diag(S) Vt.  By default blocks up to
    32 x 32 use the batched Jacobi solver and larger ones the
    polar-decomposition SVD on concurrent solver streams; ``max_sweeps`` /
    ``tol`` > 0 select one Jacobi SVD per block with that bound.  A block
    that does not converge raises QSError (QS_ERR_NUMERIC)."""
    import torch
    ctx = ctx or default_context()
    cplx = any(np.iscomplexobj(b) for b in blocks)
    dt = np.complex128 if cplx else np.float64
    es = 2 if cplx else 1
    m = np.array([b.shape[0] for b in blocks], np.int64)
    n = np.array([b.shape[1] for b in blocks], np.int64)
    k = np.minimum(m, n)
    cum = lambda x: np.concatenate([[0], np.cumsum(x)[:-1]]).astype(np.int64)  # noqa: E731
    offs, uoffs, soffs, voffs = cum(m * n), cum(m * k), cum(k), cum(k * n)
    A = np.concatenate([np.asarray(b, dt).reshape(-1, order="F") for b in blocks]) if blocks else np.zeros(0, dt)
    dev = torch.device("cuda", ctx.device)
    dA = torch.from_numpy(A.view(np.float64)).to(dev)
    dU = torch.zeros(max(int((m * k).sum()) * es, 1), dtype=torch.float64, device=dev)
    dS = torch.zeros(max(int(k.sum()), 1), dtype=torch.float64, device=dev)
    dV = torch.zeros(max(int((k * n).sum()) * es, 1), dtype=torch.float64, device=dev)
    torch.cuda.synchronize(dev)
    check(ctx.lib.qs_svd_blocks_ex(ctx.h, len(blocks), _ptr(m), _ptr(n), _ptr(offs), _ptr(uoffs), _ptr(soffs),
                                   _ptr(voffs), 1 if cplx else 0, C.c_void_p(dA.data_ptr()),
                                   C.c_void_p(dU.data_ptr()), C.c_void_p(dS.data_ptr()), C.c_void_p(dV.data_ptr()),
                                   int(max_sweeps), float(tol)))
    ctx.sync()
    U, S, V = dU.cpu().numpy(), dS.cpu().numpy(), dV.cpu().numpy()
    if cplx:
        U, V = U.view(np.complex128), V.view(np.complex128)
    Us = [U[uoffs[i]:uoffs[i] + m[i] * k[i]].reshape((m[i], k[i]), order="F") for i in range(len(blocks))]
    Ss = [S[soffs[i]:soffs[i] + k[i]] for i in range(len(blocks))]
    Vs = [V[voffs[i]:voffs[i] + k[i] * n[i]].reshape((k[i], n[i]), order="F") for i in range(len(blocks))]
    return Us, Ss, Vs


def gs_reortho(V: np.ndarray, v: np.ndarray, ctx: Context | None = None):
    """Double classical Gram-Schmidt of v against the orthonormal columns of
    V on the GPU, then normalisation.  Returns (v_new, |v| before)."""
    import torch
    ctx = ctx or default_context()
    dev = torch.device("cuda", ctx.device)
    n, nv = V.shape
    dV = torch.from_numpy(np.asfortranarray(V, np.float64).reshape(-1, order="F")).to(dev)
    dv = torch.from_numpy(np.asarray(v, np.float64).copy()).to(dev)
    torch.cuda.synchronize(dev)
    nrm = C.c_double()
    check(ctx.lib.qs_gs_reortho(ctx.h, n, nv, C.c_void_p(dV.data_ptr()), C.c_void_p(dv.data_ptr()),
                                C.byref(nrm)))
    ctx.sync()
    return dv.cpu().numpy(), nrm.value


def eigQS_dev(H, Nkeep: int = -1, Etrunc: float = 0.0, deps: float = 0.0):
    """eigQS of a device tensor (qs_eigQS_dev): the eigenvectors stay on the
    device.  Returns (Etot, I) with Etot the ascending eigenvalues of all
    blocks, I['AK'] / I['AD'] device Tensors of the kept / discarded
    eigenvectors, I['E'] the per-block eigenvalues (H's block order),
    I['keep'] their 0/1 flags, I['NK'] the reference's NK (markSet's
    min(Nkeep, N) when Etrunc > 0 and deps == 0, else the kept count; the
    kept states are the 1s of I['keep']), I['Etrunc']."""
    from .qspace import Tensor
    ctx = H.ctx
    rank, qdim, nblk, nelem, cx = H.meta()
    if rank != 2:
        raise ValueError("eigQS_dev: rank-2 tensor required")
    dims = np.empty(max(nblk * 2, 1), np.int64)
    check(ctx.lib.qs_tensor_meta(H.h, None, dims.ctypes.data_as(_capi.c_int64_p), None))
    ntot = int(dims[:2 * nblk:2].sum()) if nblk else 0
    E = np.zeros(max(ntot, 1), np.float64)
    keep = np.zeros(max(ntot, 1), np.uint8)
    ak, ad = C.c_void_p(), C.c_void_p()
    nk, et = C.c_int64(), C.c_double()
    check(ctx.lib.qs_eigQS_dev(ctx.h, H.h, int(Nkeep), float(Etrunc), float(deps), C.byref(ak), C.byref(ad),
                               E.ctypes.data_as(_capi.c_double_p), keep.ctypes.data_as(C.POINTER(C.c_uint8)),
                               C.byref(nk), C.byref(et)))
    E, keep = E[:ntot], keep[:ntot].astype(bool)
    parts = {"AK": Tensor(ctx, ak, H.info), "AD": Tensor(ctx, ad, H.info), "E": E, "keep": keep,
             "NK": nk.value, "Etrunc": et.value}
    return np.sort(E), parts



# ------------------------------------------------------------------- svdQS
# itags are strings, a trailing '*' marking an outgoing (conjugated) leg, as
# the reference prints them (itag_, Source/wbindex.hh:631-790).
def _tconj(t: str) -> str:
    return t[:-1] if t.endswith("*") else t + "*"


def _tname(t: str) -> str:
    return t[:-1] if t.endswith("*") else t


def _tdual(t: str) -> str:
    """itag_::MarkDual (Source/wbindex.cc:1125-1147): toggles a trailing
    prime on the name; names hold at most 8 characters."""
    n = _tname(t)
    n = n[:-1] if n.endswith("'") else n + "'"
    if len(n) > 8:
        raise ValueError(f"itag '{n}' longer than 8 characters")
    return n + ("*" if t.endswith("*") else "")


def _tset_(t: str, x: str) -> str:
    """itag_::Set_: an empty tag takes x; else t takes x's direction."""
    if not _tname(t):
        return x
    return _tconj(t) if t.endswith("*") != x.endswith("*") else t


def _lexsort(R: np.ndarray) -> np.ndarray:
    """Stable permutation sorting integer rows lexicographically (first
    column most significant), as wbMatrix::SortRecs (Source/wbMatrix.cc)."""
    if R.shape[0] == 0 or R.shape[1] == 0:
        return np.arange(R.shape[0])
    return np.lexsort(R.T[::-1])


def _groups(R: np.ndarray):
    """wbMatrix::groupRecs (Source/wbMatrix.cc:1733-1744): the sort
    permutation and the runs of equal rows -> (unique rows, member lists,
    group id of every row)."""
    n = R.shape[0]
    gid = np.empty(n, np.int64)
    if n == 0:
        return [], [], gid
    p = _lexsort(R)
    Rs = R[p]
    new = np.ones(n, bool)
    new[1:] = np.any(Rs[1:] != Rs[:-1], axis=1)
    starts = np.flatnonzero(new)
    gid[p] = np.cumsum(new) - 1
    return [Rs[s] for s in starts], [m.tolist() for m in np.split(p, starts[1:])], gid


class _SvdLayout:
    """Host plan of svdQS: PSI's legs permuted (the split-off legs last), its
    blocks grouped by the label sum that the SVD conserves, and every group
    laid out as one dense block matrix (rows: the distinct label records of
    the first K legs, columns: those of the rest) -- SVD_Data::blockSVD and
    QBlock::toBlockMatrix (Source/mpsortho.cc:546-613, 31-257)."""

    def __init__(self, PSI: QSpace, idx, first=None):
        """``idx``: the 1-based legs split off behind the others
        (extend2Perm(.., 'E')); or ``first``: the 1-based legs that lead,
        in the given order, the others following (extend2Perm)."""
        r = PSI.rank
        if PSI.nblk == 0:
            raise ValueError("got empty PSI")
        J = idx if first is None else first
        I = [int(i) - 1 for i in np.atleast_1d(np.asarray(J)).ravel()]
        if not I or len(I) >= r:
            raise ValueError(f"invalid index set (len={len(I)}/{r})")
        if any(i < 0 or i >= r for i in I) or len(set(I)) != len(I):
            raise ValueError("index out of bounds or not unique")
        tags = list(PSI.info.get("itags") or [])
        rest = [i for i in range(r) if i not in I]
        self.r = r
        self.P, self.K = (rest + I, r - len(I)) if first is None else (I + rest, len(I))
        K, P = self.K, self.P
        self.tags = [tags[p] for p in P] if len(tags) == r else []
        if K != 1:
            # only ingoing legs may be fused into the outgoing bond; the other
            # group must point one way (blockSVD, Source/mpsortho.cc:557-573)
            if not self.tags:
                raise ValueError("got invalid orthonormalization (rank mismatch of itags)")
            qd = [not t.endswith("*") for t in self.tags]
            if not all(qd[:K]):
                raise ValueError("got invalid orthonormalization "
                                 "(only ingoing indices can be fused into outgoing)")
            if any(q != qd[K] for q in qd[K + 1:]):
                raise ValueError("got invalid orthonormalization (2nd/right group is mixed in+out)")
        n, qdim = PSI.nblk, PSI.qdim
        Q = [np.asarray(PSI.Q[p], np.int64).reshape(n, qdim) for p in P]
        dims = [tuple(PSI.block_dims(i)[p] for p in P) for i in range(n)]
        self.qdim, self.cplx = qdim, PSI.is_complex
        Ib = [0] if K == 1 else ([K] if K == r - 1 else list(range(K)))
        qsum = sum(Q[j] for j in Ib)
        uq, members, _ = _groups(qsum)
        self.groups, self.mats = [], []
        dt = np.complex128 if self.cplx else np.float64
        for g, blks in zip(uq, members):
            R1 = np.concatenate([Q[j][blks] for j in range(K)], axis=1)
            R2 = np.concatenate([Q[j][blks] for j in range(K, r)], axis=1)
            u1, _, g1 = _groups(R1)
            u2, _, g2 = _groups(R2)
            s1 = [None] * len(u1)
            s2 = [None] * len(u2)
            seen = set()
            for b, i1, i2 in zip(blks, g1, g2):
                if (i1, i2) in seen:
                    raise ValueError("block not unique (degenerate records)")
                seen.add((i1, i2))
                for s, i, d in ((s1, i1, dims[b][:K]), (s2, i2, dims[b][K:])):
                    if s[i] is None:
                        s[i] = d
                    elif s[i] != d:
                        raise ValueError("block size mismatch")
            o1 = np.concatenate([[0], np.cumsum([int(np.prod(d)) for d in s1])]).astype(np.int64)
            o2 = np.concatenate([[0], np.cumsum([int(np.prod(d)) for d in s2])]).astype(np.int64)
            M = np.zeros((int(o1[-1]), int(o2[-1])), dt)
            for b, i1, i2 in zip(blks, g1, g2):
                blk = np.asarray(PSI.data[b]).reshape(PSI.block_dims(b), order="F").transpose(P)
                M[o1[i1]:o1[i1 + 1], o2[i2]:o2[i2 + 1]] = blk.reshape((o1[i1 + 1] - o1[i1], -1), order="F")
            # the label of the new bond: that of the single split-off leg,
            # else the label sum of U's legs (QBlock::init_bare_refA,
            # Source/mpsortho.cc:277-296); it equals the group's sum except
            # for rank 2 with both legs pointing the same way
            # (a group whose split-off leg carries several labels is refused
            # once a value of it is kept)
            mixed = r - K == 1 and any(not np.array_equal(x, u2[0]) for x in u2)
            if r - K == 1:
                g = u2[0]
            self.groups.append({"q": np.asarray(g), "rows": (u1, s1, o1), "cols": (u2, s2, o2), "mixed": mixed})
            self.mats.append(M)

    def decompose(self, Us, Ss, Vts, Nkeep=-1, Nkmin=0, stol=None, itag="", with_s=True):
        """Truncation (svd_keep) and the QSpaces U (the first K legs and the
        new bond), S (diagonal, with_s) and V (the other legs and the bond;
        with_s=False: V times S as one tensor) with their itags, before any
        final leg permutation -- SVD_Data::dmrgTruncate (Source/mpsortho.cc:
        616-905) with SQ given (svdQS) or not (orthoQS)."""
        r, K, qdim = self.r, self.K, self.qdim
        if stol is None:
            stol = 0.0 if Nkeep > 0 else 1e-8                     # WB_STOL_SVD
        Nkmin = max(int(Nkmin), 0)
        S_all = [np.asarray(s, np.float64) for s in Ss]
        keep, nk, s2t, tot, sfac = svd_keep(S_all, int(Nkeep), Nkmin, float(stol))
        SM = np.sort(np.concatenate(S_all))[::-1] if S_all else np.zeros(0)
        # the flag that dmrgTruncate reports (Source/mpsortho.cc:682-735)
        nk_u = int(Nkeep) if Nkeep >= 0 else 2 ** 32 - 1
        flag = 0
        if SM.size and SM[-1] > stol:
            if SM.size > nk_u and stol:
                flag += 1
        elif nk >= nk_u and nk < SM.size:
            flag += 1
        if s2t and tot > s2t and abs(sfac - 1) > 0.01:
            flag += 1
        info = {"svd": SM, "stol": float(stol), "svd2tr": s2t / tot if tot else 0.0, "sv2tot": tot,
                "sfac": sfac, "Nkmin": Nkmin, "Nkeep": nk, "Ntot": int(SM.size), "flag": flag, "K": K}
        # itags of U, S and Vd (Source/mpsortho.cc:737-779)
        T = self.tags
        if len(T) != r:
            raise ValueError("got invalid/empty itags")
        tu = _tname(itag or "")
        revert, i = False, -1
        if r - K == 1:
            i = r - 1
            tu = _tset_(tu, T[-1])
            if not tu.endswith("*") and nk:
                revert = not (r == 2 and T[0].endswith("*") != T[1].endswith("*"))   # iTags::isOp(2,'L')
        elif K == 1:
            i = 0
            tu = _tconj(_tset_(tu, T[0]))
        elif not T[0].endswith("*"):
            tu = _tconj(tu)
        tv = tu
        if with_s and i == 1 and r == 2:
            tu = _tname(T[0]) + ("*" if tu.endswith("*") else "")        # itag_::tSet
            if not T[1].endswith("*") and revert:
                tu = _tdual(tu)
        tU, tS, tV = T[:K] + [tu], [_tconj(tu), tv], T[K:] + [_tconj(tv)]
        # blocks: per group of kept values, U rows x new leg, S diagonal, V rows x new leg
        UQ, Ud, SQ, Sd, VQ, Vd = [], [], [], [], [], []
        for G, U, s, Vt, kp in zip(self.groups, Us, S_all, Vts, keep):
            ik = np.flatnonzero(kp)
            if ik.size == 0:
                continue
            if G["mixed"]:
                raise ValueError("got inconsistency in block symmetry")
            g = G["q"]
            Vc = np.asarray(Vt).T                                  # conj(V): PSI = U S Vc^T
            if not with_s:
                Vc = Vc * (s * sfac)[None, :]                      # Wb::DMatProd(Vc, S)
            for (u, sz, o), X, dst_q, dst_d in ((G["rows"], np.asarray(U), UQ, Ud), (G["cols"], Vc, VQ, Vd)):
                for j in range(len(u)):
                    dst_q.append(np.concatenate([u[j], g]))
                    dst_d.append(X[o[j]:o[j + 1], ik].reshape(tuple(sz[j]) + (ik.size,), order="F"))
            SQ.append(np.concatenate([g, g]))
            Sd.append((s[ik] * sfac).reshape(-1, 1))

        # the blocks of one QSpace must not repeat a label record
        # (QSpace::Append2AndDestroy 'u', Source/mpsortho.cc:806-845)
        for nm, recs in (("U", UQ), ("S", SQ if with_s else []), ("V", VQ)):
            if len({tuple(x) for x in recs}) != len(recs):
                raise ValueError(f"{nm}: QIDX must not overlap")

        def mk(recs, data, rank, tags):
            if not recs:
                return QSpace([], [], {})
            R = np.asarray(recs, np.int64).reshape(len(recs), rank, qdim)
            return QSpace([np.ascontiguousarray(R[:, k, :]).astype(np.int32) for k in range(rank)], data,
                          {"itags": tags})

        if revert:
            # U's bond and S's first leg (without S: V's bond) turn into the
            # dual (labels negated, direction flipped, primed tag); both come
            # back from the reference's identity contraction sorted by their
            # labels (Source/mpsortho.cc:867-902, QSpace::initIdentityCG 'z')
            tU[-1] = _tdual(_tconj(tU[-1]))
            if with_s:
                tS[0] = _tdual(_tconj(tS[0]))
                other = (SQ, Sd, 0)
            else:
                tV[-1] = _tdual(_tconj(tV[-1]))
                other = (VQ, Vd, (r - K) * qdim)
            for recs, data, col in ((UQ, Ud, K * qdim), other):
                for x in recs:
                    x[col:col + qdim] = -x[col:col + qdim]
                o = _lexsort(np.asarray(recs, np.int64).reshape(len(recs), -1)) if recs else []
                recs[:] = [recs[j] for j in o]
                data[:] = [data[j] for j in o]
        Sq = mk(SQ, Sd, 2, tS) if with_s else None
        return mk(UQ, Ud, K + 1, tU), Sq, mk(VQ, Vd, r - K + 1, tV), info

    def finish(self, Us, Ss, Vts, Nkeep=-1, Nkmin=0, stol=None, itag="", permA=None, permB=None):
        """svdQS's U, S, Vd and info: decompose() and svdQS's final
        permutations (Source/svdQS.cc:209-229): Vd gets its bond first; a
        single split-off leg leaves U in PSI's leg order, a single kept leg
        Vd; then permA / permB."""
        r, K, P = self.r, self.K, self.P
        _check_perms(r, permA, permB)
        Uq, Sq, Vq, info = self.decompose(Us, Ss, Vts, Nkeep, Nkmin, stol, itag, True)
        iP = list(np.argsort(P))
        n = r - K + 1
        pb = [n - 1] + list(range(n - 1))                          # wbperm::initLastTo(0, n)
        if _perm0(permB) is not None:
            pb = _compose(pb, _perm0(permB))
        pa = _perm0(permA)
        if K + 1 == r:
            pa = _compose(iP, pa) if pa is not None else iP
        elif K == 1:
            pb = _compose(iP, pb)
        if pa is not None:
            Uq = _permute(Uq, pa)
        Vq = _permute(Vq, pb)
        return Uq, Sq, Vq, info


def _check_perms(r: int, permA, permB):
    """The MEX's check of the permA / permB options (Source/svdQS.cc:192-193,
    Source/orthoQS.cc:218-219)."""
    la = 0 if permA is None else np.size(permA)
    lb = 0 if permB is None else np.size(permB)
    if la > r or lb > r or (la and lb and la + lb != r + 2):
        raise ValueError(f"invalid permutations perm[AB] (lengths {la}, {lb}; rank {r})")


def _compose(base: list, p: list) -> list:
    """wbperm::Permute (Source/wbperm.cc:538-588): both extended by the
    identity to the longer length, entry i becomes base[p[i]] for the first
    len(p) entries, the others stay."""
    n = max(len(base), len(p))
    if sorted(p) != list(range(len(p))):
        raise ValueError(f"invalid permutation {[j + 1 for j in p]}")
    ext = list(base) + list(range(len(base), n))
    return [ext[j] for j in p] + ext[len(p):]


def _perm0(p):
    """A 1-based permutation option as a 0-based list; None for an identity
    of any length (the reference skips those)."""
    if p is None:
        return None
    q = [int(x) - 1 for x in np.atleast_1d(np.asarray(p)).ravel()]
    return None if q == list(range(len(q))) else q


def _permute(A: QSpace, p: list) -> QSpace:
    """Leg permutation of a host QSpace (new leg i = old leg p[i]); the block
    order stays (QSpace::Permute, Source/QSpace.hh:2669-2719)."""
    if A.nblk == 0 or p == list(range(len(p))):
        return A
    if len(p) > A.rank or sorted(p) != list(range(len(p))):
        raise ValueError(f"permutation {[j + 1 for j in p]} out of bounds (rank {A.rank})")
    p = list(p) + list(range(len(p), A.rank))                 # a shorter one acts on the leading legs
    tags = A.info.get("itags")
    data = [np.asarray(d).reshape(A.block_dims(i), order="F").transpose(p) for i, d in enumerate(A.data)]
    return QSpace([A.Q[j] for j in p], data, {"itags": [tags[j] for j in p]} if tags else {})


def svdQS(PSI: QSpace, idx, Nkeep: int = -1, Nkmin: int = 0, stol: float | None = None, itag: str = "",
          permA=None, permB=None, ctx: Context | None = None):
    """[U, S, Vd, info] = svdQS(PSI, idx, ...) for abelian QSpaces
    (Source/svdQS.cc:170-234): the legs ``idx`` (1-based) are split off into
    Vd, the others stay with U, PSI = U * S * Vd.  The blocks of one
    conserved label sum form one matrix; all of them are decomposed in one
    call on the GPU (qs_svd_blocks_ex), truncated together
    (qs_svd_keep: Nkeep, Nkmin, stol; stol defaults to 1e-8 without Nkeep)
    with the kept values rescaled to PSI's norm.  itags, block order and the
    direction of the new bond follow the reference.  ``info`` holds svd (all
    singular values, descending), stol, svd2tr, sv2tot, sfac, Nkmin, Nkeep
    (kept count), Ntot, flag and K."""
    L = _SvdLayout(PSI, idx)
    Us, Ss, Vts = svd_blocks(L.mats, ctx)
    return L.finish(Us, Ss, Vts, Nkeep, Nkmin, stol, itag, permA, permB)


_LRDIR = {">>": 3, "<<": -3, "LR": 2, "RL": -2, "+": 1, "-": -1}


def _nkeep_estimate(L: "_SvdLayout", PSI: QSpace) -> int:
    """get_Nkeep_estimate (Source/orthoQS.cc:35-52), abelian: the smaller of
    the products of the total leg dimensions either side of the split."""
    tot = []
    for p in L.P:
        seen = {}
        for i in range(PSI.nblk):
            seen.setdefault(tuple(np.asarray(PSI.Q[p][i]).ravel()), PSI.block_dims(i)[p])
        tot.append(sum(seen.values()))
    return int(min(np.prod(tot[:L.K]), np.prod(tot[L.K:])))


class _OrthoPlan:
    """Host plan of orthoQS (Source/orthoQS.cc:156-310, usages #1 and #2):
    which legs lead the SVD, the block matrices (_SvdLayout) and the final
    leg permutations of A1 and A2."""

    def __init__(self, PSI: QSpace, idx, lrdir=None, permA=None, permB=None):
        r = PSI.rank
        I = [int(i) for i in np.atleast_1d(np.asarray(idx)).ravel()]
        if lrdir is None:
            if len(I) != 1:
                raise ValueError("orthoQS: invalid usage #1 (one index required without lrdir)")
            ldir = None
        else:
            # the MEX takes lrdir as a string only (Source/orthoQS.cc:76-79)
            ldir = _LRDIR.get(lrdir) if isinstance(lrdir, str) else None
            if not ldir:
                raise ValueError(f"orthoQS: invalid lrdir {lrdir!r}")
            if not I or len(I) >= r:
                raise ValueError(f"orthoQS: invalid index set ({len(I)}/{r})")
            if abs(ldir) == 3 and (len(I) == 1 or len(I) + 1 == r):
                I = [i for i in range(1, r + 1) if i not in I]       # ctrIdx::Invert
                ldir = -ldir
        # ldir >= 0: the legs I lead (K = len(I)); < 0: they go behind
        self.L = L = _SvdLayout(PSI, None, first=I) if (ldir is None or ldir >= 0) else _SvdLayout(PSI, I)
        self.nkeep_est = _nkeep_estimate(L, PSI)
        K, P = L.K, L.P
        iP = [int(x) for x in np.argsort(P)]
        _check_perms(r, permA, permB)
        pa_u, pb_u = _perm0(permA), _perm0(permB)
        self.swap = ldir is not None and ldir < 0
        if ldir is None:
            pa, pb = None, _compose([r - 1] + list(range(r - 1)), iP)
        elif ldir >= 0:
            pb = [r - K] + list(range(r - K))                      # initLastTo(0, r-K+1)
            if pb_u is not None:
                pb = _compose(pb, pb_u)
            pa = pa_u
            if K + 1 == r:
                pa = _compose(iP, pa) if pa is not None else iP
            elif K == 1:
                pb = _compose(iP, pb)
        else:
            n = len(I)
            pa, pb = pa_u, None
            if n + 1 == r:
                pa = _compose([n] + list(range(n)), iP)
                if pa_u is not None:
                    pa = _compose(pa, pa_u)
            elif n == 1:
                pb = _compose(iP, pb_u) if pb_u is not None else iP
            if pb is None:
                pb = [K] + list(range(K))
                if pb_u is not None:
                    pb = _compose(pb, pb_u)
        self.pa, self.pb = pa, pb

    def finish(self, Us, Ss, Vts, Nkeep=-1, Nkmin=0, stol=None, itag=""):
        if Nkeep is None or Nkeep < 0:
            Nkeep = self.nkeep_est
            if stol is None:
                stol = 1e-8
        U, _, VS, info = self.L.decompose(Us, Ss, Vts, Nkeep, Nkmin, stol, itag, with_s=False)
        A1, A2 = (VS, U) if self.swap else (U, VS)
        if self.pa is not None:
            A1 = _permute(A1, self.pa)
        return A1, _permute(A2, self.pb), info


def orthoQS(PSI: QSpace, idx, lrdir=None, Nkeep: int = -1, Nkmin: int = 0, stol: float | None = None,
            itag: str = "", permA=None, permB=None, ctx: Context | None = None):
    """[A1, A2, info] = orthoQS(PSI, idx [, lrdir], ...) for abelian QSpaces
    (Source/orthoQS.cc:156-310, usages #1 and #2): PSI = A1 * A2 through a
    new bond, A1 the isometry.  Without lrdir ``idx`` is one leg, split off
    into A1 (its leg and the bond); A2 = V S keeps PSI's leg order with the
    bond in that leg's place.  With lrdir ('>>' 'LR' '+' / '<<' 'RL' '-') the legs ``idx`` go to A1 (>=0) or to A2 (<0; '>>' / '<<' with
    one leg or all but one take the complement instead and flip the
    direction), with permA / permB applied as the reference does.  The SVD
    runs batched on the GPU; Nkeep < 0 keeps up to the smaller dimension
    either side (stol 1e-8 unless Nkeep is given)."""
    plan = _OrthoPlan(PSI, idx, lrdir, permA, permB)
    Us, Ss, Vts = svd_blocks(plan.L.mats, ctx)
    return plan.finish(Us, Ss, Vts, Nkeep, Nkmin, stol, itag)
