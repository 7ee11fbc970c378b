"""Output-block sharding of one grouped contraction (qspace_gb300.shard):
the greedy partition covers every block once and balances the flops; shards
carry only the operands their pairs read; and two gloo ranks, each computing
its shard with numpy's products, assemble exactly the unsharded result."""
import os
import socket

import numpy as np
import pytest

from qspace_gb300.grouped import Packed
from qspace_gb300.shard import assemble, block_flops, partition_blocks, shard
from qspace_gb300.workloads import grouped_pairs


def _batch(seed=3, npairs=60, shared=True):
    w = grouped_pairs(seed=seed, npairs=npairs, lo=2, hi=40, complex_data=True)
    blk = None
    if shared:
        # runs of pairs summing into one output block (equal M, N within a run)
        A, B, blk = [], [], []
        for p in range(npairs):
            b = p // 3
            m, n = 5 + b % 7, 3 + b % 5
            k = int(w["K"][p])
            A.append(w["A"][p][:1, :1].repeat(m, 0).repeat(k, 1) * (1 + p % 4))
            B.append(w["B"][p][:1, :1].repeat(k, 0).repeat(n, 1) * (2 - p % 3))
            blk.append(b)
        return Packed(A, B, w["afac"], blk=blk, cplx=True)
    return Packed(w["A"], w["B"], w["afac"], cplx=True)


def _oracle_blocks(pk):
    out = [np.zeros((m, n), complex) for (m, n, _) in pk.blocks]
    ids = {}
    for p in range(pk.n):
        b = ids.setdefault(int(pk.blk[p]), len(ids))
        a = pk.abuf[pk.a_off[p]:pk.a_off[p] + pk.M[p] * pk.K[p]].reshape((pk.M[p], pk.K[p]), order="F")
        bb = pk.bbuf[pk.b_off[p]:pk.b_off[p] + pk.K[p] * pk.N[p]].reshape((pk.K[p], pk.N[p]), order="F")
        out[b] += pk.afac[p] * (a @ bb)
    return out


@pytest.mark.parametrize("nranks", [1, 2, 3, 8])
def test_partition_covers_and_balances(nranks):
    pk = _batch(shared=False, npairs=200)
    f = block_flops(pk)
    parts = partition_blocks(f, nranks)
    allb = np.sort(np.concatenate(parts))
    assert np.array_equal(allb, np.arange(len(f)))
    loads = np.array([f[p].sum() for p in parts])
    # largest-first greedy: no rank exceeds the mean by more than one block
    assert loads.max() <= f.sum() / nranks + f.max() + 1e-6
    assert all(np.array_equal(x, y) for x, y in zip(parts, partition_blocks(f, nranks)))  # deterministic


def test_shard_keeps_only_referenced_operands():
    pk = _batch()
    parts = partition_blocks(block_flops(pk), 2)
    sizes = 0
    for idx in parts:
        s = shard(pk, idx)
        assert len(s.blocks) == len(idx)
        sizes += s.abuf.size + s.bbuf.size
    assert sizes == pk.abuf.size + pk.bbuf.size        # every operand block goes to one rank


def _shared_operand_batch():
    """Six output blocks; A block 0 feeds blocks 0, 2 and 5, A block 1 feeds
    blocks 1 and 3; B blocks are shared the same way."""
    rng = np.random.default_rng(21)
    M, N, K = [7, 9], [5, 4, 6], [3, 8]
    A = [rng.standard_normal((M[i], K[i])) + 1j * rng.standard_normal((M[i], K[i])) for i in range(2)]
    B = [rng.standard_normal((K[0], N[j])) + 1j * rng.standard_normal((K[0], N[j])) for j in range(3)] + \
        [rng.standard_normal((K[1], N[j])) + 1j * rng.standard_normal((K[1], N[j])) for j in range(3)]
    #        out: 0  1  2  3  4  5
    ia = np.array([0, 1, 0, 1, 0, 0])
    ib = np.array([0, 4, 1, 3, 2, 2])
    afac = rng.uniform(-1, 1, 6)
    return Packed.from_operands(A, B, ia, ib, afac, cplx=True), A, B, ia, ib


def test_shard_copies_shared_operands_to_every_rank_that_reads_them():
    pk, A, B, ia, ib = _shared_operand_batch()
    # the packed batch stores each operand block once
    assert pk.operand_bytes() == 16 * (sum(a.size for a in A) + sum(b.size for b in B))
    parts = partition_blocks(block_flops(pk), 2)
    total = 0
    for idx in parts:
        s = shard(pk, idx)
        pairs = set(int(p) for p in s.pairs)
        want = 16 * (sum(A[i].size for i in set(ia[list(pairs)].tolist()))
                     + sum(B[j].size for j in set(ib[list(pairs)].tolist())))
        assert s.operand_bytes() == want          # distinct blocks of its pairs, once each
        total += s.operand_bytes()
        # the shard computes its blocks exactly as the full batch does
        full = _oracle_blocks(pk)
        for b, x in zip(idx, _oracle_blocks(s)):
            assert np.array_equal(x, full[int(b)])
    # blocks read by both ranks' pairs are duplicated, so the ranks hold more than the batch
    assert total > pk.operand_bytes()


def _free_port():
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def _rank(rank, world, port, q):
    import torch.distributed as dist
    os.environ.update(MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port))
    dist.init_process_group("gloo", rank=rank, world_size=world)
    pk = _batch()
    parts = partition_blocks(block_flops(pk), world)
    mine = _oracle_blocks(shard(pk, parts[rank]))
    got = [None] * world
    dist.all_gather_object(got, mine)
    if rank == 0:
        full = assemble(pk, parts, got)
        ref = _oracle_blocks(pk)
        q.put(all(np.array_equal(x, y) for x, y in zip(full, ref)))
    dist.destroy_process_group()


def test_two_gloo_ranks_assemble_the_unsharded_result():
    import multiprocessing as mp
    ctx = mp.get_context("spawn")
    q = ctx.Queue()
    port = _free_port()
    ps = [ctx.Process(target=_rank, args=(r, 2, port, q)) for r in range(2)]
    for p in ps:
        p.start()
    for p in ps:
        p.join(120)
    assert all(p.exitcode == 0 for p in ps)
    assert q.get(timeout=10) is True


def _gather_rank(rank, world, port, q):
    import torch
    import torch.distributed as dist
    os.environ.update(MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port))
    dist.init_process_group("gloo", rank=rank, world_size=world)
    from qspace_gb300.shard import gather_blocks
    pk = _batch(shared=False, npairs=40)
    parts = partition_blocks(block_flops(pk), world)
    mine = np.concatenate([b.reshape(-1, order="F") for b in _oracle_blocks(shard(pk, parts[rank]))])
    out = gather_blocks(torch.from_numpy(mine.view(np.float64).copy()), parts, pk, dist, dst=0)
    if rank == 0:
        full = out.numpy().view(np.complex128)
        ref = np.concatenate([b.reshape(-1, order="F") for b in _oracle_blocks(pk)])
        q.put(bool(np.array_equal(full, ref)))
    else:
        q.put(out is None)
    dist.destroy_process_group()


def _spawn(target, world=2):
    import multiprocessing as mp
    ctx = mp.get_context("spawn")
    q = ctx.Queue()
    port = _free_port()
    ps = [ctx.Process(target=target, args=(r, world, port, q)) for r in range(world)]
    for p in ps:
        p.start()
    for p in ps:
        p.join(120)
    assert all(p.exitcode == 0 for p in ps)
    return [q.get(timeout=10) for _ in range(world)]


def test_gather_blocks_to_the_owner_over_two_gloo_ranks():
    """The exchange step of a sharded contraction: rank 0 receives every
    rank's blocks and holds the unsharded C arena, bit for bit."""
    assert all(_spawn(_gather_rank))


def _eig_rank(rank, world, port, q):
    import torch.distributed as dist
    os.environ.update(MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port))
    dist.init_process_group("gloo", rank=rank, world_size=world)
    from qspace_gb300.linalg import mark_keep
    from qspace_gb300.shard import partition_eig_blocks, sharded_mark_keep
    rng = np.random.default_rng(5)
    n = rng.integers(1, 30, size=23)
    E = []
    for k in n:                       # spectra with exact two-fold degeneracies
        e = np.sort(np.round(rng.standard_normal(int(k)), 3))
        E.append(e)
    parts = partition_eig_blocks(n, world)
    out = []
    for nkeep, etrunc, deps in ((50, 0.0, 0.0), (120, 0.0, 1e-6), (200, 1.5, 0.0), (-1, 0.8, 1e-9)):
        mine, nk, et = sharded_mark_keep([E[int(b)] for b in parts[rank]], parts, len(n), dist, nkeep, etrunc, deps)
        ref, nkr, etr = mark_keep(E, nkeep, etrunc, deps)
        out.append(nk == nkr and et == etr and all(np.array_equal(m, ref[int(b)]) for m, b in zip(mine, parts[rank])))
    q.put(all(out))
    dist.destroy_process_group()


def test_sharded_eig_truncation_agrees_with_one_process():
    """Block eigendecomposition sharded by symmetry block: after the one
    all-gather of the eigenvalues every rank's markSet keeps exactly the
    states the unsharded truncation keeps in its blocks (Nkeep, Etrunc and
    degeneracy averaging)."""
    assert all(_spawn(_eig_rank))
