"""Seeded synthetic inputs with the shapes of the benchmark workloads.

The reference ships no benchmark data; these generators build block-sparse
tensors with the stated sector structure and N(0,1) entries from
``numpy.random.default_rng(seed)``.

* ``mps_site_tensor`` -- abelian U(1)xU(1) (charge, 2Sz) MPS site tensor
  A(L, s, R) with 41 charge sectors q in [-20, 20] per bond (one 2Sz sector
  per charge, drawn from {-1, 0, 1}), sector dims round(512 exp(-q^2/50)/Z);
  rule for the rounding: sectors that round to 0 are dropped and the
  remainder goes to q = 0 so that every bond has D = 512.  The local site is
  d = 4 with (charge, 2Sz) in {(-1,0), (0,+1), (0,-1), (+1,0)}.  A block
  exists for every (L, s) whose fused (q_L + q_s, Sz_L + Sz_s) is a sector of
  R.  The reduced density matrix is contractQS(A, '12*', A, '12').
* ``grouped_pairs`` -- 2000 independent block pairs with M, N, K =
  round(exp(U(ln 8, ln 1024))), complex128 N(0,1) entries and a CG factor
  U(-1, 1) per pair; output = one block per pair.
* ``random_abelian`` -- small random abelian QSpaces for parity tests.
"""
from __future__ import annotations

import numpy as np

from .qspace import QSpace

LOCAL_FERMION_SITE = [(-1, 0), (0, 1), (0, -1), (1, 0)]


def bond_sectors(rng: np.random.Generator, D: int = 512, qmax: int = 20, width: float = 50.0):
    q = np.arange(-qmax, qmax + 1)
    w = np.exp(-q.astype(float) ** 2 / width)
    d = np.rint(D * w / w.sum()).astype(np.int64)
    sz = rng.integers(-1, 2, size=q.size)
    keep = d > 0
    q, d, sz = q[keep], d[keep], sz[keep]
    d[np.flatnonzero(q == 0)[0]] += D - int(d.sum())
    return [(int(a), int(b), int(c)) for a, b, c in zip(q, sz, d)]  # (charge, 2Sz, dim)


def mps_site_tensor(seed: int = 0, D: int = 512, complex_data: bool = False) -> QSpace:
    rng = np.random.default_rng(seed)
    L = bond_sectors(rng, D)
    R = bond_sectors(rng, D)
    rmap = {(q, s): d for q, s, d in R}
    QL, QS, QR, data = [], [], [], []
    for (ql, sl, dl) in L:
        for (qs, ss) in LOCAL_FERMION_SITE:
            key = (ql + qs, sl + ss)
            if key not in rmap:
                continue
            dr = rmap[key]
            QL.append((ql, sl))
            QS.append((qs, ss))
            QR.append(key)
            blk = rng.standard_normal((dl, 1, dr))
            if complex_data:
                blk = blk + 1j * rng.standard_normal((dl, 1, dr))
            data.append(blk)
    Q = [np.asarray(QL, np.int32), np.asarray(QS, np.int32), np.asarray(QR, np.int32)]
    return QSpace(Q, data, {"itags": ["L", "s", "R*"]})


def rank4_psi(seed: int = 0, D: int = 512, complex_data: bool = False) -> QSpace:
    """Two-site wave function psi(L, s1, s2, R) of the U(1)xU(1) chain: the
    bonds of ``mps_site_tensor`` (bond dimension D), two local fermion sites;
    a block for every (L, s1, s2) whose fused label is a sector of R, N(0,1)
    entries."""
    rng = np.random.default_rng(seed)
    L = bond_sectors(rng, D)
    R = bond_sectors(rng, D)
    rmap = {(q, s): d for q, s, d in R}
    Q = [[], [], [], []]
    data = []
    for (ql, sl, dl) in L:
        for (q1, s1) in LOCAL_FERMION_SITE:
            for (q2, s2) in LOCAL_FERMION_SITE:
                key = (ql + q1 + q2, sl + s1 + s2)
                if key not in rmap:
                    continue
                dr = rmap[key]
                for k, lab in enumerate(((ql, sl), (q1, s1), (q2, s2), key)):
                    Q[k].append(lab)
                blk = rng.standard_normal((dl, 1, 1, dr))
                if complex_data:
                    blk = blk + 1j * rng.standard_normal((dl, 1, 1, dr))
                data.append(blk)
    return QSpace([np.asarray(q, np.int32) for q in Q], data, {"itags": ["L", "s1", "s2", "R*"]})


def grouped_pairs(seed: int = 0, npairs: int = 2000, lo: int = 8, hi: int = 1024,
                  complex_data: bool = True):
    """Returns dict with M, N, K, afac arrays and lists of A (MxK), B (KxN)."""
    rng = np.random.default_rng(seed)
    dims = np.rint(np.exp(rng.uniform(np.log(lo), np.log(hi), size=(npairs, 3)))).astype(np.int64)
    afac = rng.uniform(-1.0, 1.0, size=npairs)
    A, B = [], []
    for p in range(npairs):
        M, N, K = (int(x) for x in dims[p])
        if complex_data:
            a = rng.standard_normal((M, K)) + 1j * rng.standard_normal((M, K))
            b = rng.standard_normal((K, N)) + 1j * rng.standard_normal((K, N))
        else:
            a = rng.standard_normal((M, K))
            b = rng.standard_normal((K, N))
        A.append(np.asfortranarray(a))
        B.append(np.asfortranarray(b))
    return {"M": dims[:, 0], "N": dims[:, 1], "K": dims[:, 2], "afac": afac, "A": A, "B": B,
            "complex": complex_data}


def random_abelian(rng: np.random.Generator, legs: list, nblk_max: int = 40,
                   complex_data: bool = False, density: float = 0.6, itags=None) -> QSpace:
    """Random abelian QSpace over the given leg sector tables.

    ``legs``: one list per leg of (label tuple, dim).  Blocks are a random
    subset of the label combinations (no conservation law is imposed; the
    contraction semantics do not need one)."""
    combos = [[]]
    for lg in legs:
        combos = [c + [i] for c in combos for i in range(len(lg))]
    rng.shuffle(combos)
    n = min(nblk_max, max(1, int(len(combos) * density)))
    combos = combos[:n]
    qdim = len(legs[0][0][0])
    Q = [np.zeros((n, qdim), np.int32) for _ in legs]
    data = []
    for b, c in enumerate(combos):
        shape = []
        for k, i in enumerate(c):
            lab, d = legs[k][i]
            Q[k][b] = lab
            shape.append(d)
        x = rng.standard_normal(shape)
        if complex_data:
            x = x + 1j * rng.standard_normal(shape)
        data.append(x)
    return QSpace(Q, data, {"itags": list(itags)} if itags else {})


def random_leg(rng: np.random.Generator, nsec: int = 4, dmax: int = 5, qdim: int = 1, qmax: int = 3):
    labs = set()
    while len(labs) < nsec:
        labs.add(tuple(int(x) for x in rng.integers(-qmax, qmax + 1, size=qdim)))
    return [(lab, int(rng.integers(1, dmax + 1))) for lab in sorted(labs)]


def nrg_eig_blocks(seed: int = 0, dmax: int = 700, sigma: float = 3.0):
    """Real symmetric Hamiltonian blocks of one NRG step (abelian stand-in):
    one block per (charge q in [-12, 12], 2Sz in -15..15 step 2) sector with
    dimension round(dmax exp(-(q^2 + Sz^2) / (2 sigma^2))) -- 336 blocks of
    uneven sizes 1..690, 39300 states -- entries N(0,1), symmetrised."""
    rng = np.random.default_rng(seed)
    blocks = []
    for q in range(-12, 13):
        for s2 in range(-15, 16, 2):
            d = int(round(dmax * np.exp(-(q * q + (s2 / 2.0) ** 2) / (2 * sigma * sigma))))
            if d < 1:
                continue
            x = rng.standard_normal((d, d))
            blocks.append(np.asfortranarray(0.5 * (x + x.T)))
    return blocks


def two_site_state(seed: int = 0, D: int = 512, complex_data: bool = False) -> QSpace:
    """Rank-4 all-in two-site wavefunction (L, s1, s2, R) with U(1) labels
    summing to zero: bond sectors q in [-4, 4] of dimension ~D exp(-q^2/8),
    local labels {-1, 0, 1} of dimension 1 -- the tensor that svdQS splits
    between the two sites of a DMRG sweep."""
    rng = np.random.default_rng(seed)
    dq = {q: max(1, int(round(D * np.exp(-q * q / 8.0)))) for q in range(-4, 5)}
    recs, data = [], []
    for qL in dq:
        for s1 in (-1, 0, 1):
            for s2 in (-1, 0, 1):
                qR = -(qL + s1 + s2)
                if qR not in dq:
                    continue
                shp = (dq[qL], 1, 1, dq[qR])
                x = rng.standard_normal(shp)
                recs.append((qL, s1, s2, qR))
                data.append(x + 1j * rng.standard_normal(shp) if complex_data else x)
    Q = [np.array([[r[k]] for r in recs], np.int32) for k in range(4)]
    return QSpace(Q, data, {"itags": ["L", "s1", "s2", "R"]})


def hpsi_chain(seed: int = 0, D: int = 4096, qmax: int = 30, sigma: float = 8.0):
    """Tensors of a two-site DMRG H*psi for a spin-1/2 chain with U(1)
    (2Sz) labels: environments L(a', w, a) and R(b', w, b), MPO tensors
    W(wl, s', s, wr) of bond dimension w = 5 (sectors 0 x3, +2, -2) and a
    two-site state psi(a, s1, s2, b), bonds of D states over 2Sz sectors
    q in [-qmax, qmax] with dims ~ exp(-q^2 / (2 sigma^2)).  Labels are
    conserved as a' = a - w, b = a + s1 + s2, s' = s + wl - wr, b' = b - w,
    so H*psi = L psi W W R keeps the labels of psi.  N(0,1) entries, no
    itags.  The order of the contractions:
        X1 = (L, 3; psi, 1)         -> (a', w1, s1, s2, b)
        X2 = (X1, [2 3]; W, [1 3])  -> (a', s2, b, s1', w2)
        X3 = (X2, [2 5]; W, [3 1])  -> (a', b, s1', s2', w3)
        Y  = (X3, [2 5]; R, [3 2])  -> (a', s1', s2', b')."""
    rng = np.random.default_rng(seed)
    q = np.arange(-qmax, qmax + 1)
    wq = np.exp(-q.astype(float) ** 2 / (2 * sigma * sigma))
    d = np.maximum(np.rint(D * wq / wq.sum()).astype(np.int64), 1)
    bond = {int(a): int(b) for a, b in zip(q, d)}
    wsec = {0: 3, 2: 1, -2: 1}
    spins = (-1, 1)

    def build(recs, shape_of):
        recs = sorted(recs)
        data = [rng.standard_normal(shape_of(r)) for r in recs]
        Q = [np.array([[r[k]] for r in recs], np.int32) for k in range(len(recs[0]))]
        return QSpace(Q, data, {})

    env = [(ap, w, a) for a in bond for w in wsec for ap in (a - w,) if ap in bond]
    Lq = build(env, lambda r: (bond[r[0]], wsec[r[1]], bond[r[2]]))
    Rq = build(env, lambda r: (bond[r[0]], wsec[r[1]], bond[r[2]]))
    ps = [(a, s1, s2, a + s1 + s2) for a in bond for s1 in spins for s2 in spins if a + s1 + s2 in bond]
    psi = build(ps, lambda r: (bond[r[0]], 1, 1, bond[r[3]]))
    wt = [(wl, sp, s, wr) for wl in wsec for wr in wsec for s in spins for sp in spins if sp == s + wl - wr]
    W = build(wt, lambda r: (wsec[r[0]], 1, 1, wsec[r[3]]))
    return Lq, psi, W, Rq
