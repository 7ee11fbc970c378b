"""A two-site DMRG H*psi chain (L psi W W R, spin-1/2, U(1) 2Sz labels) as
four device-resident contractions, plain FP64 and split, against the same
chain through the oracle's numpy contractQS: identical labels, block order
and shapes; data within 1e-13 (FP64) / 1e-11 (split)."""
import pytest

from oracle import qs_oracle as orc
from qspace_gb300 import upload
from qspace_gb300.qspace import contract_dev
from qspace_gb300.workloads import hpsi_chain
from tests.helpers import assert_qspace_close

pytestmark = pytest.mark.gpu


def _oracle_chain(L, P, W, R):
    x = orc.contract(L.to_dict(), 3, P.to_dict(), 1)
    x = orc.contract(x, [2, 3], W.to_dict(), [1, 3])
    x = orc.contract(x, [2, 5], W.to_dict(), [3, 1])
    return orc.contract(x, [2, 5], R.to_dict(), [3, 2])


@pytest.mark.parametrize("prec,tol", [("fp64", 1e-13), ("split", 1e-11)])
def test_hpsi_chain_matches_oracle(ctx, prec, tol):
    L, P, W, R = hpsi_chain(1, 512)
    ref = _oracle_chain(L, P, W, R)
    tL, tP, tW, tR = (upload(x, ctx) for x in (L, P, W, R))
    x1 = contract_dev(tL, "3", tP, "1", prec=prec)
    x2 = contract_dev(x1, "23", tW, "13", prec=prec)
    x3 = contract_dev(x2, "25", tW, "31", prec=prec)
    y = contract_dev(x3, "25", tR, "32", prec=prec)
    got = y.download()
    for t in (x1, x2, x3, y, tL, tP, tW, tR):
        t.free()
    assert got.nblk == P.nblk
    assert_qspace_close(got, ref, tol)
