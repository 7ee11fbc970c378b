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


# ------------------------------------------------------------------ exchange
def gather_blocks(local, parts: list, pk: Packed, pg, dst: int = 0):
    """The one exchange of a sharded contraction: every rank's flat buffer of
    output blocks (its shard's C arena, in ascending block order) goes to
    rank `dst`, which returns the flat C arena of the whole batch in
    pk.blocks order; the other ranks return None.  `local` is a torch tensor
    (on the GPU with NCCL, on the CPU with gloo) of the rank's doubles.
    Ranks send exactly their own blocks: no reduction, no padding copies on
    the receiving side beyond one staging buffer per rank."""
    import torch
    rank, world = pg.get_rank(), pg.get_world_size()
    cm = 2 if pk.cplx else 1
    sizes = [int(sum(pk.blocks[int(b)][0] * pk.blocks[int(b)][1] for b in p)) * cm for p in parts]
    if local.numel() != sizes[rank]:
        raise ValueError(f"rank {rank} holds {local.numel()} doubles, its blocks need {sizes[rank]}")
    mx = max(sizes) if sizes else 0
    send = local
    if local.numel() < mx:
        send = torch.zeros(mx, dtype=local.dtype, device=local.device)
        send[:local.numel()] = local
    bufs = [torch.empty(mx, dtype=local.dtype, device=local.device) for _ in range(world)] if rank == dst else None
    pg.gather(send, gather_list=bufs, dst=dst)
    if rank != dst:
        return None
    out = torch.empty(pk.c_elems * cm, dtype=local.dtype, device=local.device)
    for r, p in enumerate(parts):
        o = 0
        for b in p:
            m, n, off = pk.blocks[int(b)]
            out[off * cm:(off + m * n) * cm] = bufs[r][o:o + m * n * cm]
            o += m * n * cm
    return out


# ------------------------------------------------------------ sharded eigQS
def partition_eig_blocks(n, nranks: int) -> list:
    """Symmetry blocks per rank for a sharded block eigendecomposition:
    largest cost n^3 first onto the least-loaded rank (the eigQS loop over
    blocks, Source/QSpace.cc:4789-4811, split across GPUs)."""
    return partition_blocks(np.asarray(n, float) ** 3, nranks)


def sharded_mark_keep(local_E: list, parts: list, nblk: int, pg, nkeep: int = -1, etrunc: float = 0.0,
                      deps: float = 0.0):
    """markSet over all ranks' eigenvalues (Source/gathered.cc:1822-1990):
    each rank holds the ascending eigenvalues of its blocks (parts[rank], in
    that order); one all-gather of the eigenvalues gives every rank the whole
    spectrum in the global block order, and every rank runs the same
    truncation, so all ranks agree on NK and on each block's kept states.
    Returns (keep flags of the local blocks, NK, Etrunc)."""
    import torch

    from .linalg import mark_keep
    rank, world = pg.get_rank(), pg.get_world_size()
    mine = np.concatenate([np.asarray(e, np.float64) for e in local_E]) if local_E else np.zeros(0)
    cnt = torch.tensor([mine.size], dtype=torch.int64)
    got = [torch.zeros(1, dtype=torch.int64) for _ in range(world)]
    pg.all_gather(got, cnt)
    sizes = [int(x.item()) for x in got]
    mx = max(max(sizes), 1)
    send = torch.zeros(mx, dtype=torch.float64)
    send[:mine.size] = torch.from_numpy(mine)
    bufs = [torch.zeros(mx, dtype=torch.float64) for _ in range(world)]
    pg.all_gather(bufs, send)
    # lengths of every block, known to all ranks from the partition and the
    # gathered counts
    lens = [None] * nblk
    for r, p in enumerate(parts):
        if r == rank:
            for b, e in zip(p, local_E):
                lens[int(b)] = len(e)
    lt = torch.tensor([lens[int(b)] if lens[int(b)] is not None else -1 for b in range(nblk)], dtype=torch.int64)
    lg = [torch.zeros(nblk, dtype=torch.int64) for _ in range(world)]
    pg.all_gather(lg, lt)
    L = torch.stack(lg).max(dim=0).values.numpy()
    E_all = [None] * nblk
    for r, p in enumerate(parts):
        o = 0
        v = bufs[r].numpy()
        for b in p:
            E_all[int(b)] = v[o:o + L[int(b)]]
            o += int(L[int(b)])
    keep, nk, et = mark_keep(E_all, nkeep, etrunc, deps)
    return [keep[int(b)] for b in parts[rank]], nk, et
