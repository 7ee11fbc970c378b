"""One grouped contraction split over ranks by output block.

The pairs of different output blocks are independent: the reference runs
the per-output-block loop of contractDATA_group (Source/QSpace_aux.cc:27-355)
for every block inside one OpenMP loop (Source/QSpace.cc:4375-4393).  So a
contraction splits over R ranks with no reduction.  Each rank computes whole
output blocks from only the A/B blocks its pairs reference.  Blocks go
largest first to the least-loaded rank (flop-balanced greedy; ties go to the
lower rank, so every rank computes the same partition).  Results come back
as whole blocks.  Gathering them, when one process needs all of C, is the
only exchange.
"""
from __future__ import annotations

import numpy as np

from .grouped import Packed


def block_flops(pk: Packed) -> np.ndarray:
    """FP64-equivalent flops of each output block (sum over its pairs), in
    the order of pk.blocks."""
    per_pair = (8.0 if pk.cplx else 2.0) * pk.M.astype(float) * pk.N * pk.K
    ids = {}
    for p in range(pk.n):
        ids.setdefault(int(pk.blk[p]), len(ids))
    out = np.zeros(len(ids))
    for p in range(pk.n):
        out[ids[int(pk.blk[p])]] += per_pair[p]
    return out


def partition_blocks(flops, nranks: int) -> list:
    """Output-block indices per rank: largest block first onto the rank with
    the least work so far (ties: lower rank).  Each rank's list is ascending."""
    if nranks < 1:
        raise ValueError("nranks must be >= 1")
    f = np.asarray(flops, float)
    load = np.zeros(nranks)
    parts = [[] for _ in range(nranks)]
    for b in sorted(range(len(f)), key=lambda i: (-f[i], i)):
        r = int(np.argmin(load))
        parts[r].append(b)
        load[r] += f[b]
    return [np.array(sorted(p), np.int64) for p in parts]


def shard(pk: Packed, blocks) -> Packed:
    """The sub-batch of the pairs of output blocks `blocks` (indices into
    pk.blocks), in their original order, with only the A and B blocks those
    pairs read, each stored once even when several of its pairs read it.  An
    operand block read by output blocks of several ranks is copied to each of
    them.  Its output blocks are the selected ones, in ascending order; its
    ``pairs`` attribute holds the selected pairs' indices in pk."""
    want = set(int(b) for b in blocks)
    first = {}
    for p in range(pk.n):
        first.setdefault(int(pk.blk[p]), len(first))
    sel = [p for p in range(pk.n) if first[int(pk.blk[p])] in want]
    # distinct operand blocks by their place in pk's arenas
    amap, bmap, A, B = {}, {}, [], []
    for p in sel:
        ka = (int(pk.a_off[p]), int(pk.M[p]), int(pk.K[p]))
        if ka not in amap:
            amap[ka] = len(A)
            A.append(pk.abuf[ka[0]:ka[0] + ka[1] * ka[2]].reshape((ka[1], ka[2]), order="F"))
        kb = (int(pk.b_off[p]), int(pk.K[p]), int(pk.N[p]))
        if kb not in bmap:
            bmap[kb] = len(B)
            B.append(pk.bbuf[kb[0]:kb[0] + kb[1] * kb[2]].reshape((kb[1], kb[2]), order="F"))
    ia = [amap[(int(pk.a_off[p]), int(pk.M[p]), int(pk.K[p]))] for p in sel]
    ib = [bmap[(int(pk.b_off[p]), int(pk.K[p]), int(pk.N[p]))] for p in sel]
    out = Packed.from_operands(A, B, ia, ib, pk.afac[sel], blk=pk.blk[sel], cplx=pk.cplx)
    out.pairs = np.array(sel, np.int64)
    return out


def assemble(pk: Packed, parts: list, results: list) -> list:
    """The full list of output blocks (pk.blocks order) from each rank's
    blocks: parts[r] as returned by partition_blocks, results[r] the blocks
    its shard computed (in ascending block order)."""
    out = [None] * len(pk.blocks)
    for idx, res in zip(parts, results):
        if len(idx) != len(res):
            raise ValueError("a rank returned the wrong number of blocks")
        for b, x in zip(idx, res):
            out[int(b)] = x
    if any(x is None for x in out):
        raise ValueError("an output block was computed by no rank")
    return out
