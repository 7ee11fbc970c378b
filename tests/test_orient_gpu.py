"""Output blocks that the split path computes transposed (C^T = op(B)^T op(A)^T,
chosen when that pads the 128-row tiles much less) or, for complex data,
with the real form duplicating B instead of A: every transpose /
conjugation flag of both operands, real and complex, several pairs summing
into one block, and output blocks stored with a leading dimension larger than
their row count.  Results are checked against numpy (split: 1e-12 relative,
FP64 path: 1e-14); the untouched gaps between the blocks stay zero."""
import ctypes as C

import numpy as np
import pytest

from qspace_gb300 import _capi
from qspace_gb300._capi import PairList, Stats, check
from qspace_gb300.qspace import make_opts

pytestmark = pytest.mark.gpu


def _stored(op: np.ndarray, trans: bool, conj: bool) -> np.ndarray:
    """Storage X whose op(X) (transpose if trans, conjugate if conj) is op."""
    x = op.T if trans else op
    return np.asfortranarray(np.conj(x) if conj else x)


def _run(ctx, shapes, flags, blk, cplx, prec, pad=5, seed=0):
    rng = np.random.default_rng(seed)
    dt = np.complex128 if cplx else np.float64

    def rnd(m, n):
        x = rng.standard_normal((m, n))
        return x + 1j * rng.standard_normal((m, n)) if cplx else x

    n = len(shapes)
    opA = [rnd(m, k) for (m, n_, k) in shapes]
    opB = [rnd(k, n_) for (m, n_, k) in shapes]
    afac = rng.uniform(-2, 2, n)
    Xa = [_stored(a, bool(f & 1), bool(f & 4) and cplx) for a, f in zip(opA, flags)]
    Xb = [_stored(b, bool(f & 2), bool(f & 8) and cplx) for b, f in zip(opB, flags)]
    a_off = np.concatenate([[0], np.cumsum([x.size for x in Xa])[:-1]]).astype(np.int64)
    b_off = np.concatenate([[0], np.cumsum([x.size for x in Xb])[:-1]]).astype(np.int64)
    abuf = np.concatenate([x.reshape(-1, order="F") for x in Xa]).astype(dt)
    bbuf = np.concatenate([x.reshape(-1, order="F") for x in Xb]).astype(dt)
    # output blocks inside column-major panels with ldc = M + pad
    first = {}
    for p, b in enumerate(blk):
        first.setdefault(b, p)
    boff, off = {}, 0
    for b, p in first.items():
        m, n_, _ = shapes[p]
        boff[b] = off
        off += (m + pad) * n_
    cbuf = np.zeros(off, dt)
    M = np.array([s[0] for s in shapes], np.int32)
    N = np.array([s[1] for s in shapes], np.int32)
    K = np.array([s[2] for s in shapes], np.int32)
    lda = np.array([x.shape[0] for x in Xa], np.int32)
    ldb = np.array([x.shape[0] for x in Xb], np.int32)
    ldc = M + pad
    c_off = np.array([boff[b] for b in blk], np.int64)
    trans = np.array([f if cplx else f & 3 for f in flags], np.int32)
    blk32 = np.asarray(blk, np.int32)
    pl = PairList()
    pl.npairs = n
    i32, i64 = _capi.c_int32_p, _capi.c_int64_p
    pl.M, pl.N, pl.K = (x.ctypes.data_as(i32) for x in (M, N, K))
    pl.a_off, pl.b_off, pl.c_off = (x.ctypes.data_as(i64) for x in (a_off, b_off, c_off))
    pl.lda, pl.ldb, pl.ldc = (x.ctypes.data_as(i32) for x in (lda, ldb, ldc))
    pl.trans = trans.ctypes.data_as(i32)
    pl.afac = afac.ctypes.data_as(_capi.c_double_p)
    pl.c_blk = blk32.ctypes.data_as(i32)
    pl.is_complex = 1 if cplx else 0
    dbl = lambda x: x.view(np.float64).ctypes.data_as(_capi.c_double_p)
    st = Stats()
    check(ctx.lib.qs_grouped_gemm_host(ctx.h, C.byref(pl), dbl(abuf), len(abuf), dbl(bbuf), len(bbuf), dbl(cbuf),
                                       len(cbuf), C.byref(make_opts(prec, 0, 1e-12)), C.byref(st)))
    ref = np.zeros_like(cbuf)
    for p in range(n):
        m, n_, _ = shapes[p]
        view = ref[c_off[p]:c_off[p] + (m + pad) * n_].reshape((m + pad, n_), order="F")
        view[:m] += afac[p] * (opA[p] @ opB[p])
    return cbuf, ref


def _rel(x, r):
    return np.linalg.norm(x - r) / np.linalg.norm(r)


@pytest.mark.parametrize("cplx", [False, True])
@pytest.mark.parametrize("prec,tol", [("split", 1e-12), ("fp64", 1e-14)])
def test_transposed_blocks_all_flags(ctx, cplx, prec, tol):
    # wide blocks (few rows, many columns) are computed transposed; the last
    # two are tall and stay as they are
    flags = list(range(16)) if cplx else list(range(4))
    shapes = [(8 + 3 * i, 300 + 17 * i, 20 + 9 * i) for i in range(len(flags))] + [(400, 9, 33), (260, 40, 70)]
    flags += [0, 3]
    cbuf, ref = _run(ctx, shapes, flags, list(range(len(shapes))), cplx, prec, seed=len(flags))
    assert _rel(cbuf, ref) <= tol
    assert np.all(cbuf[ref == 0] == 0)   # rows between the blocks (ldc > M) are not written


@pytest.mark.parametrize("cplx", [False, True])
def test_transposed_shared_blocks(ctx, cplx):
    # pairs of different depth and flags summing into wide blocks
    shapes = [(12, 500, 40), (12, 500, 7), (12, 500, 300), (30, 260, 64), (30, 260, 1), (5, 1000, 129)]
    flags = [0, 3, 5 if cplx else 1, 10 if cplx else 2, 15 if cplx else 3, 6 if cplx else 2]
    cbuf, ref = _run(ctx, shapes, flags, [0, 0, 0, 1, 1, 2], cplx, "split", seed=3)
    assert _rel(cbuf, ref) <= 1e-12
    assert np.all(cbuf[ref == 0] == 0)


def _layout(m, n, cm=2):
    """The library's layout choice for an m x n complex block (0 plain, 1 C^T,
    2 B duplicated, 3 C^T with B duplicated), restated for picking shapes."""
    def cost(rows, cols):
        mt, nt = -(-rows // 128), -(-cols // 32)
        return 26900.0 * mt * nt + 49152.0 * mt + 10530.0 * nt
    c = [cost(m * cm, n), cost(n * cm, m), cost(m, 2 * n), cost(n, 2 * m)]
    best = min(range(4), key=lambda o: (c[o], o))
    return best if c[best] < 0.97 * c[0] else 0


def test_complex_layouts_all_flags(ctx):
    """Every real-form layout of a complex block (A or B duplicated, plain or
    transposed) under every transpose / conjugation flag, with pairs of
    different depth summing into each block."""
    base = [(64, 256, 40), (10, 64, 33), (400, 9, 70), (8, 300, 51)]
    assert sorted(_layout(m, n) for m, n, _ in base) == [0, 1, 2, 3]
    shapes, flags, blk = [], [], []
    for f in range(16):
        m, n, k = base[f % 4]
        for j, kk in enumerate((k, 1 + (k * 7) % 97)):
            shapes.append((m, n, kk))
            flags.append((f + 5 * j) % 16)
            blk.append(f)
    for prec, tol in (("split", 1e-12), ("fp64", 1e-14)):
        cbuf, ref = _run(ctx, shapes, flags, blk, True, prec, seed=11)
        assert _rel(cbuf, ref) <= tol
        assert np.all(cbuf[ref == 0] == 0)
