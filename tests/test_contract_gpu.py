"""contractQS / permuteQS parity: CUDA path (through the C-ABI) vs the oracle.

Bars: labels, block order and shapes bit-exact; data within 1e-14 relative
(plain FP64 path) and 1e-12 relative (split BF16 path), Frobenius norm over
all blocks of one result.
"""
import numpy as np
import pytest

from oracle import qs_oracle as orc
from qspace_gb300 import QSpace, contractQS, permuteQS
from qspace_gb300._capi import QSError
from qspace_gb300.workloads import mps_site_tensor, random_abelian, random_leg
from tests.helpers import assert_qspace_close, assert_same_structure

pytestmark = pytest.mark.gpu

TOL = {"fp64": 1e-14, "split": 1e-12}


@pytest.mark.parametrize("prec", ["fp64", "split"])
@pytest.mark.parametrize("seed", [0, 1, 2, 3, 4])
def test_reduced_density_matrix(ctx, seed, prec):
    A = mps_site_tensor(seed)
    R = orc.contract(A.to_dict(), "12*", A.to_dict(), "12")
    st = {}
    C = contractQS(A, "12*", A, "12", prec=prec, ctx=ctx, stats=st)
    assert_qspace_close(C, R, TOL[prec])
    assert st["launches"] >= 1
    assert C.info.get("itags") == ["R", "R*"]


def _legs(rng, n, qdim):
    return [random_leg(rng, nsec=int(rng.integers(2, 5)), dmax=6, qdim=qdim) for _ in range(n)]


CASES = [
    # (A legs, B legs as indices into a shared leg table, ia, ib, perm)
    ((0, 1, 2), (2, 3), "3", "1", None),
    ((0, 1, 2), (2, 1, 3), "2,3", "2,1", None),
    ((0, 1, 2), (1, 3, 0), "1,2", "3,1", "2,1"),
    ((0, 1, 2), (1, 3, 0), "2,1", "1,3", None),
    ((0, 1, 2), (2, 0, 3), "3,1", "1,2", "2,1"),
    ((0, 1, 2, 3), (3, 1, 4), "4,2", "1,2", "3,2,1"),
    ((0, 1), (1, 0), "1,2", "2,1", None),           # full contraction -> scalar
    ((0, 1, 2), (0, 1, 2), "123", "123", None),
    ((0, 1, 2), (3, 1), "2", "2", "3,2,1"),
]


@pytest.mark.parametrize("prec", ["fp64", "split"])
@pytest.mark.parametrize("cplx", [(False, False), (True, True), (True, False), (False, True)])
@pytest.mark.parametrize("case", range(len(CASES)))
def test_random_abelian(ctx, case, cplx, prec):
    rng = np.random.default_rng(100 + case)
    la, lb, ia, ib, perm = CASES[case]
    table = _legs(rng, 5, qdim=2)
    A = random_abelian(rng, [table[i] for i in la], complex_data=cplx[0])
    B = random_abelian(rng, [table[i] for i in lb], complex_data=cplx[1])
    for conj in ("", "*"):
        R = orc.contract(A.to_dict(), ia + conj, B.to_dict(), ib, perm)
        C = contractQS(A, ia + conj, B, ib, perm, prec=prec, ctx=ctx)
        assert_qspace_close(C, R, TOL[prec])


def test_numeric_indices_and_perm(ctx):
    rng = np.random.default_rng(7)
    t = _legs(rng, 4, qdim=1)
    A = random_abelian(rng, [t[0], t[1], t[2]])
    B = random_abelian(rng, [t[2], t[3]])
    R = orc.contract(A.to_dict(), [3], B.to_dict(), [1], [2, 1, 3])
    C = contractQS(A, [3], B, [1], [2, 1, 3], ctx=ctx)
    assert_qspace_close(C, R, 1e-14)


def test_no_matching_sectors_gives_empty(ctx):
    A = QSpace([np.array([[1]], np.int32), np.array([[2]], np.int32)], [np.ones((2, 3))])
    B = QSpace([np.array([[5]], np.int32), np.array([[2]], np.int32)], [np.ones((2, 3))])
    C = contractQS(A, "1", B, "1", ctx=ctx)
    assert C.nblk == 0
    R = orc.contract(A.to_dict(), "1", B.to_dict(), "1")
    assert len(R["data"]) == 0


def test_zero_block_dropped_for_rank3(ctx):
    # two A blocks feed two output blocks; one of them has all-zero data
    Q1 = np.array([[0], [1]], np.int32)
    A = QSpace([Q1, np.array([[0], [0]], np.int32), np.array([[3], [4]], np.int32)],
               [np.ones((2, 1, 3)), np.zeros((2, 1, 3))])
    B = QSpace([Q1, np.array([[7], [7]], np.int32)], [np.ones((2, 2)), np.ones((2, 2))])
    R = orc.contract(A.to_dict(), "1", B.to_dict(), "1")
    C = contractQS(A, "1", B, "1", ctx=ctx)
    assert len(R["data"]) == 1
    assert_qspace_close(C, R, 1e-14)


def test_zero_block_kept_for_hermitian_rank2(ctx):
    Q = np.array([[0], [1]], np.int32)
    A = QSpace([Q, Q], [np.eye(2), np.zeros((3, 3))])
    R = orc.contract(A.to_dict(), "2", A.to_dict(), "1")
    C = contractQS(A, "2", A, "1", ctx=ctx)
    assert len(R["data"]) == 2
    assert_qspace_close(C, R, 1e-14)


def test_errors(ctx):
    A = mps_site_tensor(0)
    with pytest.raises(QSError):
        contractQS(A, "1", A, "2", ctx=ctx)          # dims do not match
    with pytest.raises(QSError):
        contractQS(A, "4", A, "1", ctx=ctx)          # leg out of range
    with pytest.raises(QSError):
        contractQS(A, "1,1", A, "1,2", ctx=ctx)      # repeated leg
    with pytest.raises(QSError):
        contractQS(A, "12", A, "12", [1, 1], ctx=ctx)  # invalid perm


@pytest.mark.parametrize("cplx", [False, True])
def test_permuteQS(ctx, cplx):
    rng = np.random.default_rng(3)
    t = _legs(rng, 3, qdim=2)
    A = random_abelian(rng, t, complex_data=cplx)
    for perm in ([3, 1, 2], [2, 1, 3], [1, 2, 3]):
        for conj in (False, True):
            R = orc.permute(A.to_dict(), perm, conj)
            B = permuteQS(A, perm, conj, ctx=ctx)
            assert_same_structure(B, R)
            assert_qspace_close(B, R, 0.0)


def test_device_resident_chain(ctx):
    """rho = A'A computed with device-resident tensors, then rho*rho."""
    from qspace_gb300 import upload, contract_dev
    A = mps_site_tensor(1)
    tA = upload(A, ctx)
    t1 = contract_dev(tA, "12*", tA, "12")
    t2 = contract_dev(t1, "2", t1, "1")
    rho = orc.contract(A.to_dict(), "12*", A.to_dict(), "12")
    R2 = orc.contract(rho, "2", rho, "1")
    assert_qspace_close(t2.download(), R2, 1e-14)
