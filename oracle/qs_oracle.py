"""CPU oracle for the contractQS hot path -- TEST INFRASTRUCTURE ONLY.

This module is a plain numpy restatement of QSpace's block-sparse contraction
(``contractQS`` usage #1) and of the helper steps around it.  Only ``tests/``,
``__graft_entry__.smoke()`` and the ``cpu_baseline`` / ``--impl reference`` legs
of ``bench.py`` may import it, and only as the checker or as the timed CPU
baseline.  The product (``qspace_gb300``) never imports it.

Parity pinning: the restatement is checked against golden fixtures produced by
the reference's own C++ (``contractQS.cc`` compiled behind a fake MATLAB
runtime, see ``oracle/refshim``) -- ``tests/golden/*.npz`` with the generating
script ``tests/golden/make_golden.py``.

A QSpace is represented as a plain dict that mirrors QSpace's MATLAB struct
(``Source/QSpace.hh:3092`` ``{Q,data,info}``):

* ``Q``    -- list (one per leg) of int arrays of shape (nblk, qdim);
* ``data`` -- list of nblk numpy arrays, each the dense block (any memory
  order; values are what matter), shape = the leg dimensions (trailing
  singleton legs may be dropped, as in MATLAB);
* ``info`` -- optional dict (``itags`` list of str, ``qtype`` str).

Block order and labels are bit-exact with the reference; block data agree to
floating-point rounding (the reference uses BLAS dgemm/zgemm).
"""
from __future__ import annotations

import numpy as np

__all__ = [
    "parse_ctr_idx", "contract", "permute", "block_dims", "rank_of",
    "flops_of_contract", "skip_zero_blocks", "lexsort_rows", "plus", "svd_keep",
]


# --------------------------------------------------------------------------
# index strings
# --------------------------------------------------------------------------

def _str2idx(s: str) -> list[int]:
    """Restates ``Wb::Str2Idx`` (Source/wbio.c, compact mode 'x').

    A single run of alphanumerics with no separators is read digit by digit
    ('0'-'9' -> 0..9, 'A'-'Z' -> 10.., 'a'-'z' -> 36..); otherwise the tokens
    separated by ',', ';' or white space are read as integers; optional
    surrounding brackets are allowed.
    """
    t = s.strip()
    if t.startswith("[") and t.endswith("]"):
        t = t[1:-1]
    toks = [x for x in t.replace(",", " ").replace(";", " ").split() if x]
    if not toks:
        return []
    if len(toks) == 1 and not any(c in s for c in ",; "):
        out = []
        for c in toks[0]:
            if "0" <= c <= "9":
                out.append(ord(c) - 48)
            elif "A" <= c <= "Z":
                out.append(ord(c) - 65 + 10)
            elif "a" <= c <= "z":
                out.append(ord(c) - 97 + 36)
            else:
                raise ValueError(f"invalid contraction index '{s}'")
        return out
    return [int(x, 0) for x in toks]


def parse_ctr_idx(spec) -> tuple[list[int], bool]:
    """Contraction index -> (0-based list, conj flag).

    Restates ``ctrIdx::init`` (Source/wbindex.cc:482-540): a string such as
    '12*' / '1,2*' with trailing '*' for complex conjugation (an even number of
    '*' cancels), or a 1-based numeric vector (no conj).
    """
    if isinstance(spec, str):
        s = spec.rstrip()
        nconj = 0
        while s.endswith("*"):
            nconj += 1
            s = s[:-1].rstrip()
        if s.endswith(",") or s.endswith(";"):
            s = s[:-1]
        idx = _str2idx(s)
        if not idx:
            raise ValueError(f"empty contraction index '{spec}'")
        idx = [i - 1 for i in idx]
        if min(idx) < 0:
            raise ValueError(f"contraction index must be 1-based '{spec}'")
        if len(set(idx)) != len(idx):
            raise ValueError(f"invalid index set '{spec}'")
        return idx, bool(nconj % 2)
    idx = [int(x) for x in np.atleast_1d(spec)]
    if not idx or min(idx) < 1:
        raise ValueError("contraction index must be 1-based")
    if len(set(idx)) != len(idx):
        raise ValueError("invalid index set")
    return [i - 1 for i in idx], False


# --------------------------------------------------------------------------
# small helpers
# --------------------------------------------------------------------------

def rank_of(A: dict) -> int:
    return len(A["Q"])


def nblk_of(A: dict) -> int:
    return 0 if not A["Q"] else int(np.asarray(A["Q"][0]).shape[0])


def block_dims(A: dict, i: int) -> tuple[int, ...]:
    r = rank_of(A)
    s = tuple(int(x) for x in np.shape(A["data"][i]))
    if len(s) > r:
        if any(x != 1 for x in s[r:]):
            raise ValueError("block has more non-singleton dims than legs")
        s = s[:r]
    return s + (1,) * (r - len(s))


def qrows(A: dict, legs) -> np.ndarray:
    """(nblk, len(legs)*qdim) int64 label rows; restates getQsub
    (Source/QSpace.hh:2290-2340)."""
    n = nblk_of(A)
    if not legs:
        return np.zeros((n, 0), dtype=np.int64)
    return np.concatenate([np.asarray(A["Q"][k], dtype=np.int64).reshape(n, -1)
                           for k in legs], axis=1)


def lexsort_rows(R: np.ndarray) -> np.ndarray:
    """Permutation sorting integer rows lexicographically (first column most
    significant), as ``Wb::recCompare`` with lex=1 (Source/gathered.hh:538)."""
    if R.shape[0] == 0:
        return np.zeros(0, dtype=np.int64)
    if R.shape[1] == 0:
        return np.arange(R.shape[0])
    return np.lexsort(R.T[::-1])


def _match_index(QA: np.ndarray, QB: np.ndarray):
    """All (ia, ib) with identical records; restates ``matchIndex``
    (Source/wbMatrix.cc:2075) and ``Wb::matchSortedIdx`` (Source/wbsort.cc:
    154-272): sort both, merge, cross product of equal groups."""
    if QA.shape[0] == 0 or QB.shape[0] == 0:
        return np.zeros(0, np.int64), np.zeros(0, np.int64)
    pa = lexsort_rows(QA)
    pb = lexsort_rows(QB)
    Ia, Ib = [], []
    ia = ib = 0
    na, nb = len(pa), len(pb)
    while ia < na and ib < nb:
        ra, rb = tuple(QA[pa[ia]]), tuple(QB[pb[ib]])
        if ra < rb:
            ia += 1
            continue
        if ra > rb:
            ib += 1
            continue
        ja = ia
        while ja < na and tuple(QA[pa[ja]]) == ra:
            ja += 1
        jb = ib
        while jb < nb and tuple(QB[pb[jb]]) == rb:
            jb += 1
        for x in range(ia, ja):
            for y in range(ib, jb):
                Ia.append(pa[x])
                Ib.append(pb[y])
        ia, ib = ja, jb
    return np.asarray(Ia, np.int64), np.asarray(Ib, np.int64)


def _data_size(A: dict) -> int:
    return int(sum(np.size(d) for d in A["data"]))


# --------------------------------------------------------------------------
# zero-block rules
# --------------------------------------------------------------------------

def _is_hconj_rank2(Q: list, data: list, eps: float = 1e-14) -> bool:
    """Abelian ``isHConj`` for a rank-2 QSpace (Source/QSpace.cc:1719-1775,
    ``isSym_aux`` 1802-): label set invariant under leg swap, unique, and each
    block equal to the conjugate transpose of its partner within
    eps*max(1,norm)."""
    n = Q[0].shape[0]
    R = np.concatenate([Q[0], Q[1]], axis=1)
    R2 = np.concatenate([Q[1], Q[0]], axis=1)
    p1 = lexsort_rows(R)
    p2 = lexsort_rows(R2)
    if not np.array_equal(R[p1], R2[p2]):
        return False
    S = R[p1]
    if n > 1 and np.any(np.all(S[1:] == S[:-1], axis=1)):
        return False
    nrm = np.sqrt(sum(float(np.vdot(d, d).real) for d in data))
    deps = max(nrm, 1.0) * eps
    ip2 = np.empty(n, np.int64)
    ip2[p2] = np.arange(n)
    for i in range(n):
        j = p1[ip2[i]]
        if j < i:
            continue
        di, dj = np.asarray(data[i]), np.asarray(data[j])
        di = di.reshape(di.shape + (1,) * (2 - di.ndim))
        dj = dj.reshape(dj.shape + (1,) * (2 - dj.ndim))
        if di.shape != dj.shape[::-1]:
            return False
        if np.max(np.abs(di - np.conj(dj.T)), initial=0.0) > deps:
            return False
    return True


def _is_blockdiag_d(Q: list, data: list) -> bool:
    """``isBlockDiagMatrix('d')`` for rank 2 (Source/QSpace.cc:1604-1642):
    equal labels on both legs and every block stored as a vector."""
    if not np.array_equal(Q[0], Q[1]):
        return False
    for d in data:
        s = np.shape(d)
        s = tuple(s) + (1,) * (2 - len(s))
        if len(s) != 2 or (s[0] != 1 and s[1] != 1):
            return False
    return True


def skip_zero_blocks(Q: list, data: list) -> tuple[list, list]:
    """Restates ``SkipZeroData`` with eps=0 (Source/QSpace.cc:3201-3269):
    exactly-zero blocks are removed, except for a rank-2 QSpace that is
    block-diagonal in 'd' storage or hermitian, where they are kept."""
    r = len(Q)
    if not data:
        return Q, data
    keep_all = False
    if r == 2:
        if _is_blockdiag_d(Q, data) or _is_hconj_rank2(Q, data):
            keep_all = True
    if keep_all:
        return Q, data
    keep = [i for i, d in enumerate(data) if np.any(np.asarray(d) != 0)]
    if len(keep) == len(data):
        return Q, data
    Q2 = [q[keep] for q in Q]
    return Q2, [data[i] for i in keep]


# --------------------------------------------------------------------------
# contraction
# --------------------------------------------------------------------------

def _co_sort(A, ica, B, icb):
    """``if (!ica.isSorted() && !icb.isSorted())`` -> sort by the larger
    tensor (Source/QSpace.cc:4344-4349); only changes the order of the
    contracted multi-index, not the result."""
    if ica == sorted(ica) or icb == sorted(icb):
        return ica, icb
    if _data_size(A) > _data_size(B):
        o = np.argsort(ica, kind="stable")
    else:
        o = np.argsort(icb, kind="stable")
    return [ica[i] for i in o], [icb[i] for i in o]


def contract(A: dict, ia, B: dict, ib, perm=None, return_plan: bool = False):
    """C = contractQS(A, ia, B, ib [,perm]) for abelian QSpaces.

    Follows ``contract_plain`` (Source/contractQS.cc:505-594),
    ``CONTRACT_QS`` (:596-632), ``QSpace::contract`` (Source/QSpace.cc:
    4296-4420), ``contract_getIdxSet`` (:4131-4294) and the abelian branch of
    ``contractDATA_group`` (Source/QSpace_aux.cc:27-355, ``afac=1``).
    ``perm`` is 1-based over the output legs (string or sequence).
    """
    ica, conja = parse_ctr_idx(ia)
    icb, conjb = parse_ctr_idx(ib)
    ra, rb = rank_of(A), rank_of(B)
    # conjugation / itag sequence of QSpace::contract (see _conj_sequence)
    ica_s, icb_s = _co_sort(A, ica, B, icb)
    A, conja = _conj_sequence_operand(A, ica_s, conja, front_first=True)
    B, conjb = _conj_sequence_operand(B, icb_s, conjb, front_first=False)
    conja = _itag_conj_rule(A, ica_s, conja, B, icb_s, conjb)
    if nblk_of(A) == 0 or nblk_of(B) == 0:
        return _empty_like(0)
    qdA = np.asarray(A["Q"][0]).reshape(nblk_of(A), -1).shape[1]
    qdB = np.asarray(B["Q"][0]).reshape(nblk_of(B), -1).shape[1]
    if qdA != qdB:
        raise ValueError("incompatible objects (QDIM)")
    if len(ica) != len(icb):
        raise ValueError("invalid contraction (length mismatch)")
    if max(ica) >= ra or max(icb) >= rb:
        raise ValueError("index out of bounds")
    ica, icb = _co_sort(A, ica, B, icb)
    ika = [k for k in range(ra) if k not in ica]
    ikb = [k for k in range(rb) if k not in icb]
    rc = len(ika) + len(ikb)
    P = _parse_perm(perm, rc)
    info = {}
    it_a = (A.get("info") or {}).get("itags")
    it_b = (B.get("info") or {}).get("itags")
    if it_a and it_b:
        def cj(t, c):
            if not c:
                return t
            return t[:-1] if t.endswith("*") else t + "*"
        tags = [cj(it_a[k], conja) for k in ika] + [cj(it_b[k], conjb) for k in ikb]
        if P is not None:
            tags = [tags[P[k]] for k in range(rc)]
        info["itags"] = tags

    QAc, QAk = qrows(A, ica), qrows(A, ika)
    QBc, QBk = qrows(B, icb), qrows(B, ikb)
    Ia, Ib = _match_index(QAc, QBc)
    if len(Ia) == 0:
        return {"Q": [], "data": [], "info": info}
    QC = np.concatenate([QAk[Ia], QBk[Ib]], axis=1)
    if rc:
        p = lexsort_rows(QC)
        Ia, Ib, QC = Ia[p], Ib[p], QC[p]
        newgrp = np.ones(len(QC), bool)
        newgrp[1:] = np.any(QC[1:] != QC[:-1], axis=1)
        starts = np.flatnonzero(newgrp)
    else:
        starts = np.array([0])
    ends = np.append(starts[1:], len(Ia))

    out_data = []
    pairs = []
    for g, (s, e) in enumerate(zip(starts, ends)):
        acc = None
        for t in range(s, e):
            a = np.asarray(A["data"][Ia[t]]).reshape(block_dims(A, Ia[t]), order="A")
            b = np.asarray(B["data"][Ib[t]]).reshape(block_dims(B, Ib[t]), order="A")
            for i, (ka, kb) in enumerate(zip(ica, icb)):
                if a.shape[ka] != b.shape[kb]:
                    raise ValueError("contracted dimension mismatch")
            if conja:
                a = np.conj(a)
            if conjb:
                b = np.conj(b)
            c = np.tensordot(a, b, axes=(ica, icb))
            acc = c if acc is None else acc + c
            pairs.append((g, int(Ia[t]), int(Ib[t])))
        out_data.append(np.asarray(acc))
    qdim = qdA
    Qout = [QC[starts, k * qdim:(k + 1) * qdim].astype(np.int32) for k in range(rc)]

    # SkipZeroData inside QSpace::contract, then Permute, then again.
    Qout, out_data = skip_zero_blocks(Qout, out_data)
    if P is not None and rc:
        Qout = [Qout[P[k]] for k in range(rc)]
        out_data = [np.transpose(d.reshape(d.shape + (1,) * (rc - d.ndim)), P)
                    for d in out_data]
    Qout, out_data = skip_zero_blocks(Qout, out_data)
    C = {"Q": Qout, "data": out_data, "info": info}
    if return_plan:
        return C, {"ica": ica, "icb": icb, "pairs": pairs}
    return C


def _conj_sequence_operand(X: dict, ic: list, conj: bool, front_first: bool):
    """permute_to (Source/QSpace.hh:2824-2866): an operand whose contracted
    legs are neither leading nor trailing in pairing order is permuted; its
    conjugation flag goes into that permutation, which conjugates the data
    and the itags, and the flag is cleared.  Returns (operand, conj flag)."""
    r, n = rank_of(X), len(ic)
    in_place = ic == list(range(n)) or ic == list(range(r - n, r))
    if in_place or not conj:
        return X, conj
    Y = dict(X)
    Y["data"] = [np.conj(np.asarray(d)) for d in X["data"]]
    tags = (X.get("info") or {}).get("itags")
    if tags:
        Y["info"] = dict(X.get("info") or {})
        Y["info"]["itags"] = [t[:-1] if t.endswith("*") else t + "*" for t in tags]
    return Y, False


def _itag_conj_rule(A, ica, conja, B, icb, conjb) -> bool:
    """itag check of contract_getIdxSet (Source/QSpace.cc:4230-4271) with
    itag_::sameAs (Source/wbindex.cc:989-1005): contracted legs must carry
    the same name, all with the same relative direction; if all point the
    same way and the conj flags do not differ, A is conjugated."""
    ta = (A.get("info") or {}).get("itags")
    tb = (B.get("info") or {}).get("itags")
    if not ta or not tb:
        return conja
    zflag = 0
    for a, b in zip(ica, icb):
        na, nb = ta[a].rstrip("*"), tb[b].rstrip("*")
        if na != nb and na and nb:
            raise ValueError(f"itag mismatch {ta[a]} <> {tb[b]}")
        q = 1 if ta[a].endswith("*") == tb[b].endswith("*") else -1
        if zflag and q != zflag:
            raise ValueError("itag mismatch (mixed directions)")
        zflag = zflag or q
    if zflag > 0 and conja == conjb:
        return not conja
    return conja


def _empty_like(rc: int) -> dict:
    return {"Q": [], "data": [], "info": {}}


def _parse_perm(perm, rc):
    if perm is None or (isinstance(perm, str) and not perm.strip()):
        return None
    if isinstance(perm, str):
        p = _str2idx(perm)
    else:
        p = [int(x) for x in np.atleast_1d(perm)]
    if not p:
        return None
    p = [x - 1 for x in p]
    if sorted(p) != list(range(len(p))) or len(p) > rc:
        raise ValueError(f"invalid permutation {perm}")
    if len(p) < rc:
        p = p + list(range(len(p), rc))
    return p


def itag_pairs(ta: list, ca: bool, tb: list, cb: bool):
    """Legs that an itag (cell) contraction pairs up: iTags::getCtr
    (Source/wbindex.cc:1512-1595) with itag_::sameAs (:989-1007).  Same name
    and opposite direction, or the same direction when exactly one operand
    carries a conj flag; if nothing matches the other polarity is used and
    A's conj flag toggles.  Returns (ia, ib, flipA), 0-based."""
    def name(t):
        return t.split("*")[0]

    def d(t):
        return "*" in t

    cflag = ca != cb
    for it in range(2):
        q = 1 if cflag else -1
        ma, mb, nc, e = [0] * len(ta), [0] * len(tb), 0, 0
        for i, x in enumerate(ta):
            for j, y in enumerate(tb):
                if name(x) != name(y) or (1 if d(x) == d(y) else -1) != q:
                    continue
                if not ma[i] and not mb[j]:
                    ma[i], mb[j], nc = j + 1, i + 1, nc + 1
                else:
                    e += 1
        if nc or e:
            break
        cflag = not cflag
    if e:
        raise ValueError("itag contraction: non-unique itags")
    if not nc:
        raise ValueError("itag contraction: no matching itags")
    ia = [i for i in range(len(ta)) if ma[i]]
    ib = [ma[i] - 1 for i in ia]
    return ia, ib, it == 1


def contract_cell(items: list, perm=None) -> dict:
    """contractQS({X0, X1, '*', ...} [,perm]): right to left, C = X_{n-1},
    C = X_k * C over itag-matched legs (contractQS_itags, Source/contractQS.cc:
    634-808); a '*' after a QSpace is its conj option; an empty operand gives
    an empty result."""
    X = []
    for x in items:
        if isinstance(x, str):
            X[-1] = (X[-1][0], not X[-1][1])
        else:
            X.append((x, False))
    B, cb = X[-1]
    for k in range(len(X) - 2, -1, -1):
        A, ca = X[k]
        if not A["data"] or not B["data"]:
            return {"Q": [], "data": [], "info": {}}
        ia, ib, flip = itag_pairs(A["info"]["itags"], ca, B["info"]["itags"], cb)
        sa = ",".join(str(i + 1) for i in ia) + ("*" if ca != flip else "")
        sb = ",".join(str(j + 1) for j in ib) + ("*" if cb else "")
        B = contract(A, sa, B, sb, perm if k == 0 else None)
        cb = False
    return B


def permute(A: dict, perm, conj: bool = False) -> dict:
    """permuteQS(A, perm [,'conj']) for abelian QSpaces (Source/permuteQS.cc:
    198-258; ``QSpace::Permute`` Source/QSpace.hh:2670-2719): the legs of the
    labels and of every block are reordered, block order is unchanged."""
    r = rank_of(A)
    P = _parse_perm(perm, r)
    Q = [np.asarray(q) for q in A["Q"]]
    data = [np.asarray(d).reshape(block_dims(A, i)) for i, d in enumerate(A["data"])]
    if P is not None:
        Q = [Q[P[k]] for k in range(r)]
        data = [np.transpose(d, P) for d in data]
    if conj:
        data = [np.conj(d) for d in data]
    return {"Q": Q, "data": data, "info": dict(A.get("info") or {})}


def plus(A: dict, B: dict, bfac: float = 1.0) -> dict:
    """Restates plusQS for abelian QSpaces (Source/plusQS.cc:11-45 ->
    QSpace::plus_plain, Source/QSpace.cc:3593-3700; getQOverlapU :3520-):
    the label records of A then B are concatenated and grouped (groupRecs:
    lexicographic order, a record at most once per operand); each output
    block is A's block + bfac * B's block (either alone when the other has
    none), then SkipZeroData."""
    na, nb = nblk_of(A), nblk_of(B)
    if na == 0 and nb == 0:
        return {"Q": [], "data": [], "info": dict(A.get("info") or B.get("info") or {})}
    r = rank_of(A) if na else rank_of(B)
    rows, src = [], []
    for X, tag, n in ((A, 0, na), (B, 1, nb)):
        if n:
            rows.append(qrows(X, list(range(r))))
            src += [(tag, i) for i in range(n)]
    R = np.concatenate(rows, axis=0)
    P = lexsort_rows(R)
    cplx = any(np.iscomplexobj(d) for X in (A, B) for d in X["data"])
    dt = np.complex128 if cplx else np.float64
    outQ, data = [], []
    k = 0
    while k < len(P):
        e = k + 1
        while e < len(P) and np.array_equal(R[P[e]], R[P[k]]):
            e += 1
        if e - k > 2 or (e - k == 2 and src[P[k]][0] == src[P[k + 1]][0]):
            raise ValueError("plus: non-unique block labels")
        acc = None
        for j in range(k, e):
            tag, i = src[P[j]]
            X = B if tag else A
            blk = np.asarray(X["data"][i], dt).reshape(block_dims(X, i), order="F") * (bfac if tag else 1.0)
            acc = blk if acc is None else acc + blk
        outQ.append(R[P[k]])
        data.append(acc)
        k = e
    Rq = np.asarray(outQ)
    qd = Rq.shape[1] // r
    Q = [Rq[:, l * qd:(l + 1) * qd].astype(np.int32) for l in range(r)]
    Q, data = skip_zero_blocks(Q, data)
    info = dict(A.get("info") or {}) or dict(B.get("info") or {})
    if not data:
        return {"Q": [], "data": [], "info": info}
    return {"Q": Q, "data": data, "info": info}


def flops_of_contract(A: dict, ia, B: dict, ib) -> int:
    """FP64-equivalent flops of one contraction: 2*M*N*K per real pair,
    8*M*N*K per complex pair, summed over all block pairs."""
    _, plan = contract(A, ia, B, ib, return_plan=True)
    ica, icb = plan["ica"], plan["icb"]
    tot = 0
    cplx = any(np.iscomplexobj(d) for d in A["data"]) or any(np.iscomplexobj(d) for d in B["data"])
    for (_, a, b) in plan["pairs"]:
        da, db = block_dims(A, a), block_dims(B, b)
        K = int(np.prod([da[k] for k in ica]))
        M = int(np.prod(da)) // max(K, 1)
        N = int(np.prod(db)) // max(K, 1)
        tot += (8 if cplx else 2) * M * N * K
    return tot


# --------------------------------------------------------------------------
# truncation (markSet) and the Gram-Schmidt step
# --------------------------------------------------------------------------

def average_levels(E_blocks: list, deps: float) -> list:
    """markSet's degeneracy averaging (Source/gathered.cc:1847-1866): all
    levels in stable ascending order, each run of consecutive levels closer
    than deps * |max - min| replaced by its mean, written back per block in
    the input order (E.permute(x, iP) and the memcpy into E0 there) -- the
    levels eigQS reports when deps > 0."""
    sizes = [len(e) for e in E_blocks]
    E = np.concatenate([np.asarray(e, float) for e in E_blocks]) if E_blocks else np.zeros(0)
    N = len(E)
    if N == 0 or not deps > 0:
        return [np.asarray(e, float).copy() for e in E_blocks]
    P = np.argsort(E, kind="stable")
    s = E[P].copy()
    eps = deps * abs(s[-1] - s[0])
    i0 = 0
    for i in range(1, N + 1):
        if i == N or abs(s[i] - s[i - 1]) > eps:
            if i - i0 > 1:
                s[i0:i] = np.mean(s[i0:i])
            i0 = i
    x = np.empty(N)
    x[P] = s
    return [x[o:o + n] for o, n in zip(np.cumsum([0] + sizes[:-1]), sizes)]


def mark_keep(E_blocks: list, nkeep: int = -1, etrunc: float = 0.0, deps: float = 0.0):
    """Kept-eigenvalue mask per block; restates markSet for ascending order
    (Source/gathered.cc:1822-2040) with eigQS's option handling
    (Source/eigQS.cc:55-100): deps > 0 averages near-degenerate levels and
    moves the cut to the largest weighted gap near Nkeep (b=-1, dmax=-1).
    Returns (list of bool arrays, the reference's NK output): NK is the
    number kept, except with Etrunc > 0 and deps = 0, where markSet leaves it
    at min(Nkeep, N) (only its gap-search branch rewrites Nkeep)."""
    sizes = [len(e) for e in E_blocks]
    E = np.concatenate([np.asarray(e, float) for e in E_blocks]) if E_blocks else np.zeros(0)
    N = len(E)
    keep = np.zeros(N, bool)
    out = lambda nk=None: ([keep[s:s + n] for s, n in zip(np.cumsum([0] + sizes[:-1]), sizes)],
                           int(keep.sum()) if nk is None else int(nk))
    if N == 0:
        return out()
    P = np.argsort(E, kind="stable")
    s = E[P].copy()
    b = -1.0 if deps > 0 else 0.0
    if deps > 0:
        eps = deps * abs(s[-1] - s[0])
        i0 = 0
        for i in range(1, N + 1):
            if i == N or abs(s[i] - s[i - 1]) > eps:
                if i - i0 > 1:
                    s[i0:i] = np.mean(s[i0:i])
                i0 = i
    Nk = N if (nkeep < 0 or nkeep > N) else nkeep
    if Nk == 0:
        return out()
    if Nk >= N and etrunc <= 0:
        keep[:] = True
        return out()
    if etrunc > 0:
        x = etrunc + s[0]
        l = 1
        while l < N and not (s[l] >= x and l > 0):
            l += 1
        l = min(l, Nk)
    else:
        l = Nk
    if 0 < l < N and b < 0:
        nx = max(16, l // 5)
        q = 10.0 / (-b * nx)
        NX = int(5.0 / q)
        i = max(1, l - NX)
        i2 = min(N, l + NX)
        imax, xmax = l, 0.0
        while i < i2:
            t = q * (i - l)
            x = np.exp(-t * t) * abs(s[i] - s[i - 1])
            if x > xmax:
                xmax, imax = x, i
            i += 1
        if i == N:
            t = q * (i - l)
            x = 0.1 * np.exp(-t * t) * abs(s[N - 1] - s[0])
            if x > xmax:
                xmax, imax = x, i
        l = imax
    keep[P[:min(l, N)]] = True
    return out(Nk if (etrunc > 0 and not deps > 0) else None)


def svd_keep(S_blocks: list, nkeep: int = -1, nkmin: int = 0, stol: float = 0.0):
    """Restates the truncation of svdQS: SVD_Data::dmrgTruncate
    (Source/mpsortho.cc:616-700) with markSet in descending mode
    (Source/gathered.cc:1822-1880, 1964-1972, 2037-2090; eps = b = 0).  All
    singular values sorted ascending (stable); with stol > 0 the cut l is the
    highest index with S[l] <= stol below N - Nkmin; the kept states are those
    above the cut, at most Nkeep; the kept values are then rescaled by
    sfac = sqrt(sum S^2 / (sum S^2 - discarded S^2)).  Returns (per-block
    keep flags, number kept, discarded weight s2t, total weight, sfac)."""
    sizes = [len(x) for x in S_blocks]
    E0 = np.concatenate([np.asarray(x, float) for x in S_blocks]) if S_blocks else np.zeros(0)
    N = len(E0)
    keep = np.zeros(N, bool)
    nkmin = max(0, int(nkmin))
    if N:
        P = np.argsort(E0, kind="stable")
        E = E0[P]
        nk = N if nkeep < 0 else int(nkeep)
        if nk == 0:
            pass
        elif nk >= N and stol <= 0:
            keep[:] = True
        else:
            nk = min(nk, N)
            if stol > 0:
                lx = N - nkmin if nkmin < N else 0
                l = None
                for j in range(N - 1, -1, -1):
                    if E[j] <= stol and j < lx:
                        l = j
                        break
                if l is None:
                    l = N - 1 - nk if N > nk else None
                elif N - 1 - l > nk:
                    l = N - 1 - nk
            else:
                l = N - 1 - nk
            if l is None or l < 0:
                keep[:] = True
            elif l < N - 1:
                keep[P[l + 1:]] = True
    s2 = E0 ** 2
    snorm2 = float(s2.sum())
    s2t = float(s2[~keep].sum())
    sfac = float(np.sqrt(snorm2 / (snorm2 - s2t))) if 0 < s2t < snorm2 else 1.0
    offs = np.concatenate([[0], np.cumsum(sizes)]).astype(int)
    return [keep[offs[i]:offs[i + 1]] for i in range(len(sizes))], int(keep.sum()), s2t, snorm2, sfac


def gs_reortho(V: np.ndarray, v: np.ndarray):
    """Double classical Gram-Schmidt of v against the orthonormal columns of
    V, then normalisation (Source/david2SiteQS.cc:440-470).  Returns
    (v_new, |v| before normalisation)."""
    v = np.array(v, dtype=float)
    for _ in range(2):
        if V.shape[1]:
            v = v - V @ (V.T @ v)
    n = float(np.linalg.norm(v))
    return (v / n if n > 0 else v * 0.0), n
