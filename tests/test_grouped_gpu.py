"""Grouped block products (qs_grouped_gemm*): plain FP64 and split BF16 paths
vs numpy FP64 products, including tile edges and accumulator drains."""
import numpy as np
import pytest

from qspace_gb300 import grouped
from qspace_gb300.workloads import grouped_pairs

pytestmark = pytest.mark.gpu


def numpy_ref(w):
    return [w["afac"][p] * (w["A"][p] @ w["B"][p]) for p in range(len(w["M"]))]


def rel(C, R):
    num = sum(float(np.sum(np.abs(c - r) ** 2)) for c, r in zip(C, R))
    den = sum(float(np.sum(np.abs(r) ** 2)) for r in R)
    return np.sqrt(num / den)


@pytest.mark.parametrize("cplx", [False, True])
@pytest.mark.parametrize("prec,tol", [("fp64", 1e-14), ("split", 1e-12)])
def test_grouped_small(ctx, cplx, prec, tol):
    w = grouped_pairs(seed=5, npairs=40, lo=1, hi=300, complex_data=cplx)
    C = grouped.run_host(w, prec=prec, ctx=ctx)
    assert rel(C, numpy_ref(w)) <= tol


@pytest.mark.parametrize("shape", [(1, 1, 1), (7, 9, 5), (128, 64, 32), (129, 65, 33), (127, 63, 31),
                                   (256, 200, 17), (300, 10, 700), (5, 300, 1100), (64, 64, 2000)])
@pytest.mark.parametrize("cplx", [False, True])
def test_split_edges(ctx, shape, cplx):
    """Tile and K-block edges, and depths beyond one accumulator chunk."""
    M, N, K = shape
    rng = np.random.default_rng(M * 1000 + N * 10 + K)
    a = rng.standard_normal((M, K))
    b = rng.standard_normal((K, N))
    if cplx:
        a = a + 1j * rng.standard_normal((M, K))
        b = b + 1j * rng.standard_normal((K, N))
    w = {"M": np.array([M]), "N": np.array([N]), "K": np.array([K]), "afac": np.array([0.75]),
         "A": [np.asfortranarray(a)], "B": [np.asfortranarray(b)], "complex": cplx}
    C = grouped.run_host(w, prec="split", ctx=ctx)
    assert rel(C, numpy_ref(w)) <= 1e-12
    C64 = grouped.run_host(w, prec="fp64", ctx=ctx)
    assert rel(C64, numpy_ref(w)) <= 1e-14


@pytest.mark.parametrize("cplx", [False, True])
def test_split_large_accumulators(ctx, cplx):
    """Operands whose digits all carry the same sign and nearly full size:
    every accumulator chunk sums to beyond 2^22, close to the 2^24 bound of
    exact FP32 accumulation that sets the chunk depth; products of constant
    blocks come out exact."""
    M, N, K = 200, 72, 900
    a = np.full((M, K), 0.9990234375)          # 1023/1024: top digits near full size
    b = np.full((K, N), -0.998046875)
    if cplx:
        a = a + 1j * a
        b = b - 1j * b
    w = {"M": np.array([M]), "N": np.array([N]), "K": np.array([K]), "afac": np.array([1.0]),
         "A": [np.asfortranarray(a)], "B": [np.asfortranarray(b)], "complex": cplx}
    C = grouped.run_host(w, prec="split", ctx=ctx)
    R = numpy_ref(w)
    assert rel(C, R) <= 1e-15
    assert np.array_equal(C[0], R[0])


def test_split_wide_dynamic_range(ctx):
    """Rows and columns spanning many binades: per-row/column scales."""
    rng = np.random.default_rng(11)
    M, N, K = 96, 80, 150
    a = rng.standard_normal((M, K)) * np.exp2(rng.integers(-40, 40, size=(M, 1)))
    b = rng.standard_normal((K, N)) * np.exp2(rng.integers(-40, 40, size=(1, N)))
    w = {"M": np.array([M]), "N": np.array([N]), "K": np.array([K]), "afac": np.array([1.0]),
         "A": [np.asfortranarray(a)], "B": [np.asfortranarray(b)], "complex": False}
    C = grouped.run_host(w, prec="split", ctx=ctx)[0]
    R = numpy_ref(w)[0]
    # error relative to each output element's own scale |a_i||b_j|
    scale = np.abs(a).max(axis=1)[:, None] * np.abs(b).max(axis=0)[None, :] * K
    assert np.max(np.abs(C - R) / scale) <= 1e-14


@pytest.mark.parametrize("nslices", [3, 4])
def test_split_fewer_slices_report_error(ctx, nslices):
    """3- and 4-digit products: error stated, well above 1e-12 but bounded."""
    w = grouped_pairs(seed=2, npairs=20, lo=8, hi=256, complex_data=True)
    st = {}
    C = grouped.run_host(w, prec="split", nslices=nslices, ctx=ctx, stats=st)
    e = rel(C, numpy_ref(w))
    assert st["nslices"] == nslices
    assert e <= 50 * st["err_bound"] + 1e-15
    assert e > 1e-15


def test_multi_pair_blocks_with_distinct_factors(ctx):
    """Several pairs summed into one output block with different CG factors
    (factors folded into the digits of A)."""
    rng = np.random.default_rng(4)
    M, N = 70, 90
    Ks = [33, 100, 7, 260]
    A = [np.asfortranarray(rng.standard_normal((M, k))) for k in Ks]
    B = [np.asfortranarray(rng.standard_normal((k, N))) for k in Ks]
    af = np.array([0.5, -1.25, 3.0, 1e-3])
    ref = sum(f * (a @ b) for f, a, b in zip(af, A, B))
    for prec, tol in (("fp64", 1e-14), ("split", 1e-12)):
        C = grouped.run_host_blocks(A, B, af, blk=[0, 0, 0, 0], prec=prec, ctx=ctx)
        assert rel([C[0]], [ref]) <= tol


def test_device_api_matches_host_api(ctx):
    w = grouped_pairs(seed=9, npairs=30, lo=8, hi=200, complex_data=True)
    Ch = grouped.run_host(w, prec="split", ctx=ctx)
    Cd = grouped.run_device(w, prec="split", ctx=ctx)
    for a, b in zip(Ch, Cd):
        assert np.array_equal(a, b)
