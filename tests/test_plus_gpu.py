"""plusQS on device tensors (qs_plus_dev) against the oracle's restatement of
QSpace::plus_plain: union of the label sets in lexicographic order, A + bfac B
on shared blocks, real + complex, SkipZeroData (a cancelled block disappears;
the rank-2 hermitian exemption keeps it), mismatched dims refused."""
import numpy as np
import pytest

from oracle import qs_oracle as orc
from qspace_gb300 import QSpace
from qspace_gb300._capi import QSError
from qspace_gb300.qspace import plusQS

pytestmark = pytest.mark.gpu


def _rand_qspace(rng, labels, cplx, rank=3, dims=None):
    Q = [np.array([[l[2 * k], l[2 * k + 1]] for l in labels], np.int32) for k in range(rank)]
    data = []
    for l in labels:
        shp = dims[tuple(l)] if dims else tuple(int(rng.integers(1, 6)) for _ in range(rank))
        x = rng.standard_normal(shp)
        data.append(x + 1j * rng.standard_normal(shp) if cplx else x)
    return QSpace(Q, data, {})


def _close(C: QSpace, R: dict, tol=1e-15):
    assert C.nblk == len(R["data"])
    for k in range(C.rank):
        assert np.array_equal(np.asarray(C.Q[k]).reshape(C.nblk, -1), np.asarray(R["Q"][k]).reshape(C.nblk, -1))
    for x, y in zip(C.data, R["data"]):
        x, y = np.asarray(x), np.asarray(y).reshape(np.shape(x), order="F") if np.size(y) == np.size(x) else y
        assert np.max(np.abs(x - y)) <= tol * max(1.0, np.max(np.abs(y)))


@pytest.mark.parametrize("ca,cb", [(False, False), (False, True), (True, False), (True, True)])
def test_plus_matches_oracle(ctx, ca, cb):
    rng = np.random.default_rng(3)
    la = [tuple(int(v) for v in rng.integers(-2, 3, 6)) for _ in range(12)]
    la = list(dict.fromkeys(la))
    lb = la[::3] + [tuple(int(v) for v in rng.integers(-2, 3, 6)) for _ in range(8)]
    lb = list(dict.fromkeys(lb))
    dims = {l: tuple(int(v) for v in rng.integers(1, 6, 3)) for l in set(la) | set(lb)}
    A = _rand_qspace(rng, la, ca, dims=dims)
    B = _rand_qspace(rng, lb, cb, dims=dims)
    for bfac in (1.0, -0.75):
        C = plusQS(A, B, bfac, ctx=ctx)
        R = orc.plus(A.to_dict(), B.to_dict(), bfac)
        _close(C, R)


def test_plus_cancellation_and_rank2_exemption(ctx):
    rng = np.random.default_rng(4)
    lab = [(0, 1, 0, 1, 2, 0), (1, 0, 1, 0, 0, 0)]
    A = _rand_qspace(rng, lab, False)
    C = plusQS(A, A, -1.0, ctx=ctx)                  # every block cancels
    assert C.nblk == 0
    # rank 2, block diagonal and hermitian: a cancelled block is kept
    H = QSpace([np.array([[0], [1]], np.int32)] * 2, [np.eye(2), np.full((3, 3), 2.0)], {})
    G = QSpace([np.array([[1]], np.int32)] * 2, [np.full((3, 3), 1.0)], {})
    C = plusQS(H, G, -2.0, ctx=ctx)
    R = orc.plus(H.to_dict(), G.to_dict(), -2.0)
    assert C.nblk == 2 and len(R["data"]) == 2
    _close(C, R)


def test_plus_rejects_mismatched_dims(ctx):
    A = QSpace([np.array([[0]], np.int32)] * 2, [np.ones((2, 3))], {})
    B = QSpace([np.array([[0]], np.int32)] * 2, [np.ones((3, 2))], {})
    with pytest.raises(QSError) as e:
        plusQS(A, B, ctx=ctx)
    assert e.value.code == 2
