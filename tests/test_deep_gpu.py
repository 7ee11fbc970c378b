"""Deep output blocks (a few output tiles, a very deep summed K -- reduced
density matrices and overlaps over large bonds): the grouped products cut
such a block along its depth into parts computed as blocks of their own and
summed in a fixed order (qspace_gb300/csrc/qs_deep.cu).  The results match
numpy's FP64 products on both paths (transposed operands, CG factors,
pairs cut in the middle, blocks of ordinary depth beside them), a
contraction with a deep block gives the same bits alone and in a batch, and
the reduced density matrix of a large-bond site tensor matches the FP64
path."""
import numpy as np
import pytest

from qspace_gb300 import contract_batch, contract_dev, upload
from qspace_gb300.grouped import DeviceBatch, Packed
from qspace_gb300.workloads import mps_site_tensor
from tests.helpers import assert_qspace_close

pytestmark = pytest.mark.gpu


def _rel(C, R):
    num = sum(float(np.sum(np.abs(c - r) ** 2)) for c, r in zip(C, R))
    den = sum(float(np.sum(np.abs(r) ** 2)) for r in R)
    return float(np.sqrt(num / den))


def _batch(cplx, seed):
    rng = np.random.default_rng(seed)
    def m(r, c):
        x = rng.standard_normal((r, c))
        return x + 1j * rng.standard_normal((r, c)) if cplx else x
    shapes = [  # (M, N, K, block): blocks 0 and 2 are deep, 1 is ordinary
        (5, 7, 70000, 0), (5, 7, 3, 0), (5, 7, 20011, 0),
        (64, 64, 64, 1),
        (40, 3, 50000, 2),
        (9, 2, 1, 3), (9, 2, 9000, 3),
    ]
    A = [m(M, K) for M, N, K, _ in shapes]
    B = [m(K, N) for M, N, K, _ in shapes]
    afac = rng.uniform(-1, 1, len(shapes))
    blk = [b for *_, b in shapes]
    return A, B, afac, blk


def _transpose_some(pk, A, B, which):
    """Stores op(A) of the listed pairs transposed (A^T, lda = K) and op(B)
    transposed (B^T, ldb = N): trans bits 1 and 2."""
    dt = pk.abuf.dtype
    abufs, bbufs, ao, bo, a0, b0 = [], [], [], [], 0, 0
    for p in range(pk.n):
        a = np.asarray(A[p], dt)
        b = np.asarray(B[p], dt)
        if p in which:
            a, b = a.T, b.T
            pk.trans[p] = 3
            pk.lda[p] = max(a.shape[0], 1)
            pk.ldb[p] = max(b.shape[0], 1)
        abufs.append(a.reshape(-1, order="F"))
        bbufs.append(b.reshape(-1, order="F"))
        ao.append(a0)
        bo.append(b0)
        a0 += a.size
        b0 += b.size
    pk.abuf, pk.bbuf = np.concatenate(abufs), np.concatenate(bbufs)
    pk.a_off, pk.b_off = np.array(ao, np.int64), np.array(bo, np.int64)


@pytest.mark.parametrize("cplx", [False, True])
@pytest.mark.parametrize("prec,tol", [("fp64", 1e-13), ("split", 1e-12)])
def test_grouped_deep_blocks(ctx, cplx, prec, tol):
    A, B, afac, blk = _batch(cplx, 5 + int(cplx))
    pk = Packed(A, B, afac, blk=blk, cplx=cplx)
    _transpose_some(pk, A, B, {2, 4})
    ref = {}
    for p, b in enumerate(blk):
        ref[b] = ref.get(b, 0) + afac[p] * (A[p] @ B[p])
    db = DeviceBatch(pk, ctx)
    db.dC.fill_(float("nan"))
    db.run(prec)
    got = db.result()
    R = [ref[b] for b in sorted(ref)]
    assert _rel(got, R) <= tol
    for g, r in zip(got, R):      # every block, the ordinary one too
        assert _rel([g], [r]) <= tol


@pytest.mark.parametrize("prec", ["fp64", "split"])
def test_rdm_of_large_bond_tensor(ctx, prec):
    """rho(s, s') = sum over both bonds of A(L,s,R) A*(L,s',R), D = 4096: each
    output block sums ~10^5 products."""
    A = upload(mps_site_tensor(seed=3, D=4096, complex_data=True), ctx)
    rho = contract_dev(A, "13", A, "13*", prec=prec).download()
    ref = contract_dev(A, "13", A, "13*", prec="fp64").download()
    host = A.download()
    # numpy: the same sum block by block
    exp = {}
    for i, d in enumerate(host.data):
        s = tuple(np.asarray(host.Q[1][i]).ravel())
        x = np.asarray(d).reshape(d.shape[0], d.shape[2], order="F") if np.ndim(d) == 3 else np.asarray(d)
        exp[s] = exp.get(s, 0) + np.vdot(x, x)
    assert len(ref.data) >= 2
    for i, d in enumerate(ref.data):
        s = tuple(np.asarray(ref.Q[0][i]).ravel())
        assert abs(np.asarray(d).ravel()[0] - exp[s]) <= 1e-12 * abs(exp[s])
    assert_qspace_close(rho, ref.to_dict(), 1e-12 if prec == "split" else 1e-14)
    A.free()


@pytest.mark.parametrize("prec", ["fp64", "split"])
def test_deep_contraction_alone_equals_batch(ctx, prec):
    A = upload(mps_site_tensor(seed=4, D=2048, complex_data=True), ctx)
    B = upload(mps_site_tensor(seed=5, D=256, complex_data=True), ctx)
    S = upload(mps_site_tensor(seed=6, D=64, complex_data=True), ctx)
    # a deep block next to ordinary ones, and (split path) next to a product
    # that reads a permuted operand in place
    jobs = [(A, "13", A, "13*", None), (B, "12*", B, "12", None), (A, "12*", A, "12", None),
            (S, "2", S, "2*", None)]
    alone = [contract_dev(a, ia, b, ib, p, prec=prec).download() for (a, ia, b, ib, p) in jobs]
    got = contract_batch(jobs, prec=prec)
    for g, r in zip(got, alone):
        G = g.download()
        assert len(G.data) == len(r.data)
        for x, y in zip(G.data, r.data):
            assert np.array_equal(x, y)


def _shallow_batch(cplx, seed):
    """Output blocks with a summed depth of at most 8: a row vector times a
    wide operand (M = 1, the application of a site operator over a leg of
    dimension 1), several shallow pairs into one block, transposed storage."""
    rng = np.random.default_rng(seed)
    def m(r, c):
        x = rng.standard_normal((r, c))
        return x + 1j * rng.standard_normal((r, c)) if cplx else x
    shapes = [(1, 300000, 1, 0), (1, 300000, 1, 0), (4, 70000, 2, 1), (4, 70000, 3, 1), (4, 70000, 3, 1),
              (70000, 3, 1, 2), (64, 64, 64, 3), (2, 2, 8, 4)]
    A = [m(M, K) for M, N, K, _ in shapes]
    B = [m(K, N) for M, N, K, _ in shapes]
    return A, B, rng.uniform(-1, 1, len(shapes)), [b for *_, b in shapes]


@pytest.mark.parametrize("cplx", [False, True])
@pytest.mark.parametrize("prec,tol", [("fp64", 1e-14), ("split", 1e-12)])
def test_grouped_shallow_blocks(ctx, cplx, prec, tol):
    A, B, afac, blk = _shallow_batch(cplx, 11 + int(cplx))
    pk = Packed(A, B, afac, blk=blk, cplx=cplx)
    _transpose_some(pk, A, B, {1, 3})
    ref = {}
    for p, b in enumerate(blk):
        ref[b] = ref.get(b, 0) + afac[p] * (A[p] @ B[p])
    db = DeviceBatch(pk, ctx)
    db.dC.fill_(float("nan"))
    db.run(prec)
    got = db.result()
    for g, r in zip(got, [ref[b] for b in sorted(ref)]):
        assert _rel([g], [r]) <= tol


@pytest.mark.parametrize("prec", ["fp64", "split"])
def test_shallow_blocks_plan_equals_one_shot(ctx, prec):
    """Reusable plans take shallow blocks the same way as the one-shot call:
    the replayed graph gives the same bits."""
    A, B, afac, blk = _shallow_batch(True, 21)
    pk = Packed(A, B, afac, blk=blk, cplx=True)
    db = DeviceBatch(pk, ctx)
    db.run(prec)
    ref = [c.copy() for c in db.result()]
    plan = db.plan(prec)
    for _ in range(2):
        db.dC.fill_(float("nan"))
        db.run_plan(plan)
        for g, r in zip(db.result(), ref):
            assert np.array_equal(g, r)
    plan.close()
