"""permuteQS kernels against numpy's transpose, block for block and bit for
bit: ranks 1..6, legs of size 1 (dropped by the host), legs that stay
adjacent (merged), tile edges of the 32 x 32 shared-memory tiles (sizes 7, 8,
31, 32, 33, 65), the fastest leg kept (output-order lines) and moved (tiles),
real and complex data with and without conjugation."""
import itertools

import numpy as np
import pytest

from qspace_gb300 import QSpace, permuteQS
from qspace_gb300.workloads import rank4_psi

pytestmark = pytest.mark.gpu


def _space(rng, shapes, cplx):
    r = len(shapes[0])
    n = len(shapes)
    Q = [np.arange(n, dtype=np.int32).reshape(n, 1) + 10 * k for k in range(r)]
    data = []
    for s in shapes:
        x = rng.standard_normal(s)
        if cplx:
            x = x + 1j * rng.standard_normal(s)
        data.append(x)
    return QSpace(Q, data, {})


def _check(ctx, A, perm, conj):
    B = permuteQS(A, [p + 1 for p in perm], conj, ctx=ctx)
    assert B.nblk == A.nblk
    for x, y in zip(A.data, B.data):
        ref = np.transpose(np.asarray(x), perm)
        if conj:
            ref = np.conj(ref)
        y = np.asarray(y).reshape(ref.shape)
        assert np.array_equal(y, ref)


@pytest.mark.parametrize("cplx", [False, True])
def test_rank3_all_permutations_tile_edges(ctx, cplx):
    rng = np.random.default_rng(1)
    shapes = [(7, 1, 8), (31, 3, 33), (32, 1, 32), (65, 2, 40), (8, 8, 8), (1, 1, 1), (33, 5, 1), (2, 70, 9)]
    A = _space(rng, shapes, cplx)
    for perm in itertools.permutations(range(3)):
        for conj in (False, True):
            _check(ctx, A, perm, conj)


@pytest.mark.parametrize("cplx", [False, True])
def test_random_ranks_up_to_six(ctx, cplx):
    rng = np.random.default_rng(2)
    for r in range(1, 7):
        for _ in range(4):
            shapes = []
            for _ in range(5):
                s = tuple(int(v) for v in rng.choice([1, 2, 3, 5, 8, 9, 17, 33], size=r))
                while np.prod(s) > 200000:
                    s = tuple(max(1, v // 2) for v in s)
                shapes.append(s)
            A = _space(rng, shapes, cplx)
            perm = tuple(int(p) for p in rng.permutation(r))
            _check(ctx, A, perm, bool(rng.integers(2)))


def test_rank4_psi_permutations(ctx):
    """The rank-4 two-site wave function (bond D = 512): the permutations a
    DMRG step applies."""
    psi = rank4_psi(seed=3, D=512)
    for perm in ((3, 1, 2, 0), (1, 2, 0, 3), (0, 3, 1, 2), (3, 2, 1, 0)):
        _check(ctx, psi, perm, False)
