"""Block eigendecomposition / SVD / Gram-Schmidt through the C-ABI.

* ``eigQS(H, Nkeep=, Etrunc=, deps=)`` mirrors the abelian use of the MEX
  ``eigQS`` (Source/eigQS.cc:27-122 -> QSpace::EigenSymmetric,
  Source/QSpace.cc:4673-4939): every symmetry block of a block-diagonal
  rank-2 QSpace is diagonalised on the GPU in FP64, the global truncation
  (markSet) keeps the Nkeep lowest levels, and the kept / discarded
  eigenvectors come back as QSpaces AK / AD with eigenvalues EK / ED.
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
    returns lists U, S, Vt with A = U diag(S) Vt.  ``max_sweeps`` / ``tol``
    bound the Jacobi iteration (0: the library defaults); a block that does
    not converge raises QSError (QS_ERR_NUMERIC)."""
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

