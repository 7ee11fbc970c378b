"""qs_grouped_gemm_host on batches large enough to be cut into chunks whose
host<->device copies overlap the products: the result equals the device-buffer
entry point's (bit for bit on the FP64 path, whose per-pair arithmetic does not
depend on the chunking), also when the pairs read A, B and write C out of
arena order (no early copy-out then)."""
import numpy as np
import pytest

from qspace_gb300 import grouped
from qspace_gb300.grouped import DeviceBatch, Packed, PinnedBatch
from qspace_gb300.workloads import grouped_pairs

pytestmark = pytest.mark.gpu


def _rel(C, R):
    num = sum(float(np.sum(np.abs(c - r) ** 2)) for c, r in zip(C, R))
    den = sum(float(np.sum(np.abs(r) ** 2)) for r in R)
    return np.sqrt(num / den)


@pytest.fixture(scope="module")
def batch():
    # ~0.5 GB of complex operands: three chunks of 128 MiB or more
    w = grouped_pairs(seed=21, npairs=400, lo=8, hi=1024, complex_data=True)
    pk = Packed(w["A"], w["B"], w["afac"], cplx=True)
    assert 16 * (len(pk.abuf) + len(pk.bbuf)) >= 3 * 128 * 2 ** 20
    return w, pk


def _host(pk, ctx, prec):
    pb = PinnedBatch(pk, ctx)
    st = {}
    pb.run(prec, 0, 1e-12, st)
    c = pb.c.numpy().view(np.complex128) if pk.cplx else pb.c.numpy()
    return pk.unpack_c(c), st


def _device(pk, ctx, prec):
    db = DeviceBatch(pk, ctx)
    db.run(prec, 0, 1e-12)
    return db.result()


def test_pipelined_fp64_equals_device_path(ctx, batch):
    w, pk = batch
    H, st = _host(pk, ctx, "fp64")
    D = _device(pk, ctx, "fp64")
    assert st["npairs"] == pk.n and st["launches"] >= 3
    for h, d in zip(H, D):
        assert np.array_equal(h, d)
    for p in (0, 7, 150, 399):
        r = w["afac"][p] * (w["A"][p] @ w["B"][p])
        assert np.linalg.norm(H[p] - r) <= 1e-14 * max(np.linalg.norm(r), 1e-300)


def test_pipelined_split_within_tolerance(ctx, batch):
    _, pk = batch
    H, st = _host(pk, ctx, "split")
    D = _device(pk, ctx, "fp64")
    assert st["nslices"] >= 2
    assert _rel(H, D) <= 1e-12


def test_pipelined_out_of_order_layout(ctx, batch):
    """Pairs visited in reverse: A/B watermarks jump to the end in the first
    chunk and the output ranges are not ordered, so C goes out once."""
    _, pk = batch
    rev = Packed([np.zeros((1, 1))], [np.zeros((1, 1))], [1.0])   # shell, filled below
    for k in ("M", "N", "K", "a_off", "b_off", "c_off", "lda", "ldb", "ldc", "trans", "afac", "blk"):
        setattr(rev, k, np.ascontiguousarray(getattr(pk, k)[::-1]))
    rev.blk = np.arange(pk.n, dtype=np.int32)
    rev.cplx, rev.n, rev.abuf, rev.bbuf, rev.c_elems = pk.cplx, pk.n, pk.abuf, pk.bbuf, pk.c_elems
    rev.blocks = [(int(m), int(n), int(o)) for m, n, o in zip(rev.M, rev.N, rev.c_off)]
    H, _ = _host(rev, ctx, "fp64")
    D = _device(pk, ctx, "fp64")
    for h, d in zip(H, D[::-1]):
        assert np.array_equal(h, d)


def test_small_batch_single_chunk_still_zero_fills(ctx):
    w = grouped_pairs(seed=2, npairs=6, lo=4, hi=40, complex_data=False)
    C = grouped.run_host(w, prec="fp64", ctx=ctx)
    for p in range(6):
        r = w["afac"][p] * (w["A"][p] @ w["B"][p])
        assert np.allclose(C[p], r, rtol=1e-14, atol=1e-13)
