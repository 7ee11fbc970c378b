"""One Wilson-chain NRG iteration on device-resident QSpaces.

The iteration of NRGWilsonQS (Source/NRGWilsonQS.cc: the loop around
:740-900 with nrgBuildH4_cg, :1197-1300) for a spinful fermion chain with
abelian U(1) charge x U(1) spin symmetry (labels (q, 2Sz); a site holds
|0> (-1,0), |up> (0,1), |dn> (0,-1), |updn> (1,0), q counting electrons
relative to half filling):

  H_{N+1} = sqrt(Lambda) H_N + t_N sum_s (f_{N,s}^+ f_{N+1,s} + h.c.)

1. A4(K, s, n): the product basis of the kept space K and the new site s,
   one identity slice per (sector of K, site state) inside the combined
   sector n = K + s (initIdentityCG for abelian symmetries).
2. H4 = A4^+ (sqrt(Lambda) HK x 1) A4 + t sum_s [A4^+ (F_s^+ Z x c_s) A4 + h.c.]
   with the kept-space annihilator F_s of the last site and the fermionic
   sign Z = (-1)^N of the kept states (carried by A4Z = Z A4): contractQS and
   plusQS on the device.  The first term is diagonal in the product basis
   (sqrt(Lambda) E_K on each slice of A4) and is laid out on the host: as a
   contraction its exactly-zero blocks (a zero-energy sector) would be
   dropped by SkipZeroData.
3. eigQS of H4 with the global truncation (markSet): the eigenvectors stay
   on the device.
4. The new A-tensor A(K, s, k) = A4 AK and the annihilator of the new site in
   the new kept basis, F'_s = A^+ (Z x c_s) A.

Everything but the label bookkeeping of A4 (host-built, uploaded) and the
eigenvalues (a few bytes per state, needed on the host for the truncation)
stays on the device.  The driver is written against a small backend
interface (``DeviceBackend`` here); any object with the same methods that
works on host QSpace dicts runs the same iteration on the CPU.
"""
from __future__ import annotations

import math
from dataclasses import dataclass, field

import numpy as np

from .qspace import QSpace

SITE_LABELS = [(-1, 0), (0, 1), (0, -1), (1, 0)]   # |0>, |up>, |dn>, |updn>


def site_ops() -> dict:
    """Annihilators of one site as rank-2 QSpaces (out, in) with 1x1 blocks;
    |updn> = c_up^+ c_dn^+ |0>, so c_dn |updn> = -|up>."""
    L = SITE_LABELS
    def op(entries):
        Q0 = np.array([L[o] for o, _, _ in entries], np.int32)
        Q1 = np.array([L[i] for _, i, _ in entries], np.int32)
        return QSpace([Q0, Q1], [np.array([[v]], np.float64) for _, _, v in entries], {})
    return {"up": op([(0, 1, 1.0), (2, 3, 1.0)]), "dn": op([(0, 2, 1.0), (1, 3, -1.0)])}


def parity(label, nsites: int) -> int:
    """(-1)^N of a sector: N = q + nsites electrons."""
    return -1 if (int(label[0]) + nsites) % 2 else 1


@dataclass
class KeptSpace:
    """The kept space after an iteration: sectors (label -> ascending
    eigenvalues of its kept states) and the last site's annihilators F_s in
    that basis (backend tensors)."""
    nsites: int
    E: dict                        # label tuple -> np.ndarray of energies
    F: dict = field(default_factory=dict)
    A: object = None               # A-tensor (K, s, k) of the last iteration (backend tensor)
    nkept: int = 0
    ntotal: int = 0                # states before truncation
    Eall: np.ndarray = None        # all energies of the iteration, ascending


def initial_space(backend, eps: float = 0.0, U: float = 0.0) -> KeptSpace:
    """Site 0 alone: H_0 = eps n + U n_up n_dn, F_s = c_s."""
    E = {}
    for lab, n_up, n_dn in zip(SITE_LABELS, (0, 1, 0, 1), (0, 0, 1, 1)):
        E[lab] = np.array([eps * (n_up + n_dn) + U * n_up * n_dn])
    ops = site_ops()
    return KeptSpace(1, E, {s: backend.put(c) for s, c in ops.items()}, nkept=4, ntotal=4)


class Packed:
    """A QSpace in packed form: labels q (nblk, rank, 2), dims (nblk, rank)
    and the blocks column-major back to back in buf -- built with whole-array
    numpy operations (the product basis of a large kept space has thousands
    of blocks) and uploaded in one piece where the backend can."""

    def __init__(self, q, dims, buf):
        self.q, self.dims, self.buf = q, dims, buf

    def qspace(self) -> QSpace:
        n, r = self.dims.shape
        sizes = np.prod(self.dims, axis=1)
        parts = np.split(self.buf, np.cumsum(sizes)[:-1]) if n else []
        data = [x.reshape(tuple(self.dims[i]), order="F") for i, x in enumerate(parts)]
        return QSpace([np.ascontiguousarray(self.q[:, k, :]) for k in range(r)], data, {})


def _put(backend, P: Packed):
    put_packed = getattr(backend, "put_packed", None)
    return put_packed(P) if put_packed else backend.put(P.qspace())


def _scatter_ones(nblk_rows, first, cols0, rows, offs):
    """Linear indices of entries (i, off + i) of column-major blocks with
    `rows` rows: block b contributes nblk_rows[b] entries, its block starts
    at offs[b] and its diagonal at column cols0[b]."""
    blk = np.repeat(np.arange(len(nblk_rows)), nblk_rows)
    i = np.arange(int(np.sum(nblk_rows))) - np.repeat(first, nblk_rows)
    return offs[blk] + i + (cols0[blk] + i) * rows[blk]


def _fusion(K: KeptSpace):
    """A4 and A4Z = Z_K A4 (packed), and the combined sectors."""
    sectors = sorted(K.E)
    off, D = {}, {}
    for s in SITE_LABELS:
        for qk in sectors:
            qn = (qk[0] + s[0], qk[1] + s[1])
            off[(qk, s)] = D.get(qn, 0)
            D[qn] = D.get(qn, 0) + len(K.E[qk])
    lab, d, dn, o, sign = [], [], [], [], []
    for s in SITE_LABELS:
        for qk in sectors:
            qn = (qk[0] + s[0], qk[1] + s[1])
            lab.append((qk, s, qn))
            d.append(len(K.E[qk]))
            dn.append(D[qn])
            o.append(off[(qk, s)])
            sign.append(parity(qk, K.nsites))
    d, dn, o = (np.array(x, np.int64) for x in (d, dn, o))
    q = np.array(lab, np.int32).reshape(len(lab), 3, 2)
    dims = np.stack([d, np.ones_like(d), dn], axis=1)
    sizes = d * dn
    offs = np.concatenate([[0], np.cumsum(sizes)[:-1]]).astype(np.int64)
    idx = _scatter_ones(d, np.concatenate([[0], np.cumsum(d)[:-1]]), o, d, offs)
    buf = np.zeros(int(sizes.sum()))
    bufz = np.zeros_like(buf)
    buf[idx] = 1.0
    bufz[idx] = np.repeat(np.array(sign, np.float64), d)
    return Packed(q, dims, buf), Packed(q.copy(), dims.copy(), bufz), D, off


def _diag_product(K: KeptSpace, D: dict, off: dict, f: float) -> Packed:
    """f (E_K x 1) in the product basis: one diagonal block per combined
    sector, E_K placed on the slice of each (K sector, site state)."""
    diag = {qn: np.zeros(dd) for qn, dd in D.items()}
    for (qk, s), o in off.items():
        qn = (qk[0] + s[0], qk[1] + s[1])
        diag[qn][o:o + len(K.E[qk])] = f * K.E[qk]
    labs = sorted(diag)
    n = np.array([D[l] for l in labs], np.int64)
    q = np.repeat(np.array(labs, np.int32).reshape(len(labs), 1, 2), 2, axis=1)
    dims = np.stack([n, n], axis=1)
    sizes = n * n
    offs = np.concatenate([[0], np.cumsum(sizes)[:-1]]).astype(np.int64)
    idx = _scatter_ones(n, np.concatenate([[0], np.cumsum(n)[:-1]]), np.zeros_like(n), n, offs)
    buf = np.zeros(int(sizes.sum()))
    buf[idx] = np.concatenate([diag[l] for l in labs]) if labs else np.zeros(0)
    return Packed(q, dims, buf)


def step(K: KeptSpace, backend, t: float, Lambda: float, nkeep: int = -1, deps: float = 0.0) -> KeptSpace:
    """One iteration: H_{N+1} from the kept space K, its eigen-decomposition
    and truncation to nkeep states (markSet; deps > 0 keeps near-degenerate
    levels together), the new kept space."""
    A4, A4Z, D, off = _fusion(K)
    a4, a4z = _put(backend, A4), _put(backend, A4Z)
    c = {s: backend.put(q) for s, q in site_ops().items()}
    H = _put(backend, _diag_product(K, D, off, math.sqrt(Lambda)))
    for s in ("up", "dn"):
        Fd = backend.permute(K.F[s], [2, 1], conj=True)            # f_{N,s}^+ in K
        X1 = backend.contract(Fd, "2", a4z, "1")                   # (K', s, n), Z on K
        X2 = backend.contract(c[s], "2", X1, "2")                  # (s', K', n)
        T = backend.contract(a4, "12*", X2, "21")                  # (n', n)
        # T + T^+ first: every partial sum stays hermitian, so SkipZeroData's
        # rank-2 exemption keeps zero-energy sectors of H
        H = backend.plus(H, backend.plus(T, backend.permute(T, [2, 1], conj=True), 1.0), t)
    labels, E, keep, AK = backend.eig(H, nkeep, deps)
    Anew = backend.contract(a4, "3", AK, "1")                      # (K, s, k)
    AnewZ = backend.contract(a4z, "3", AK, "1")
    F = {}
    for s in ("up", "dn"):
        X = backend.contract(c[s], "2", AnewZ, "2")                # (s', K, k)
        F[s] = backend.contract(Anew, "12*", X, "21")              # (k', k)
    Ek = {}
    for lab, e, k in zip(labels, E, keep):
        if np.any(k):
            Ek[lab] = e[k]
    return KeptSpace(K.nsites + 1, Ek, F, Anew, nkept=int(sum(int(np.sum(k)) for k in keep)),
                     ntotal=int(sum(len(e) for e in E)), Eall=np.sort(np.concatenate(E)))


class DeviceBackend:
    """The iteration's operations on device tensors (qs_contract_dev,
    qs_permute_dev, qs_plus_dev, qs_eigQS_dev)."""

    def __init__(self, ctx=None, prec: str = "fp64"):
        from .qspace import default_context
        self.ctx = ctx or default_context()
        self.prec = prec

    def put(self, A: QSpace):
        from .qspace import upload
        return upload(A, self.ctx)

    def put_packed(self, P: Packed):
        from .qspace import upload_packed
        return upload_packed(P.q, P.dims, P.buf, self.ctx)

    def contract(self, A, ia, B, ib):
        from .qspace import contract_dev
        return contract_dev(A, ia, B, ib, prec=self.prec)

    def permute(self, A, perm, conj=False):
        from .qspace import permute_dev
        return permute_dev(A, perm, conj)

    def plus(self, A, B, f):
        from .qspace import plus_dev
        return plus_dev(A, B, f)

    def eig(self, H, nkeep, deps=0.0):
        """(labels of H's blocks, per-block ascending energies, per-block
        kept flags, device tensor of the kept eigenvectors)."""
        from .linalg import eigQS_dev
        _, I = eigQS_dev(H, Nkeep=nkeep, deps=deps)
        I["AD"].free()
        return _split_blocks(H, I["E"], I["keep"]) + (I["AK"],)


def _split_blocks(H, E, keep):
    """Labels of H's diagonal blocks and the per-block slices of the
    eigenvalues / keep flags (given in H's block order)."""
    from . import _capi
    rank, qdim, nblk, _, _ = H.meta()
    q = np.empty(max(nblk * rank * qdim, 1), np.int32)
    dims = np.empty(max(nblk * rank, 1), np.int64)
    _capi.check(H.ctx.lib.qs_tensor_meta(H.h, q.ctypes.data_as(_capi.c_int32_p),
                                         dims.ctypes.data_as(_capi.c_int64_p), None))
    q = q[:nblk * rank * qdim].reshape(nblk, rank, qdim)
    n = dims[:nblk * rank:rank]
    o = np.concatenate([[0], np.cumsum(n)[:-1]]).astype(np.int64)
    labels = [tuple(int(x) for x in q[i, 0]) for i in range(nblk)]
    return (labels, [E[o[i]:o[i] + n[i]] for i in range(nblk)], [keep[o[i]:o[i] + n[i]] for i in range(nblk)])


class ServingBackend(DeviceBackend):
    """The iteration with its contractions and its eigQS sent as requests to
    a serving loop (qspace_gb300.serve.Server): the way many NRG runs share
    one GPU.  Uploads, permutations and sums run on the instance's own
    context; requests are submitted as that context's client
    (qs_server_submit_from), so each waits for the instance's queued work
    and its results belong to the instance's context.  Request latencies
    (submit to completion) are recorded per kind."""

    def __init__(self, server, ctx=None, prec: str = "fp64"):
        super().__init__(ctx, prec)
        self.server = server
        self.latency = {"contract": [], "eig": []}

    def contract(self, A, ia, B, ib):
        T, ms = self.server.wait(self.server.submit(A, ia, B, ib, prec=self.prec, client=self.ctx))
        self.latency["contract"].append(ms)
        return T

    def eig(self, H, nkeep, deps=0.0):
        r = self.server.wait_eig(self.server.submit_eig(H, nkeep, 0.0, deps, client=self.ctx))
        self.latency["eig"].append(r["latency_ms"])
        r["AD"].free()
        return _split_blocks(H, r["E"], r["keep"]) + (r["AK"],)


def wilson_hopping(n: int, Lam: float, z: float = 0.0) -> float:
    """Hopping t_n of the Wilson chain in the rescaled units of the
    iteration (H_{N+1} = sqrt(Lambda) H_N + t_N ...), with the z-shift of the
    logarithmic discretisation entering as Lambda^(-z/2) (z in [0, 1))."""
    a = 1.0 - Lam ** (-(n + 1))
    b = math.sqrt((1.0 - Lam ** (-(2 * n + 1))) * (1.0 - Lam ** (-(2 * n + 3))))
    return 0.5 * (1.0 + 1.0 / Lam) * a / b * Lam ** (-z / 2.0)


def kept_schedule(iters: int, first: int = 256, last: int = 4096) -> list:
    """Kept states per iteration growing geometrically from `first` to `last`."""
    if iters <= 1:
        return [last]
    return [int(round(first * (last / first) ** (i / (iters - 1)))) for i in range(iters)]
