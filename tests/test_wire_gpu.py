"""Device tensors through the wire container: a container uploads with one
host->device copy (qs_tensor_from_wire) and a device tensor writes one
(qs_tensor_to_wire).  Chained through device contractions, the results equal
the host API's bit for bit and the reference's golden outputs within 1e-14;
an uploaded container written back is byte-identical."""
import json
from pathlib import Path

import numpy as np
import pytest

from qspace_gb300 import QSpace, contractQS
from qspace_gb300.qspace import contract_dev, from_wire, to_wire, upload_wire
from tests.golden.golden_io import unpack
from tests.helpers import assert_qspace_close

pytestmark = pytest.mark.gpu
G = Path(__file__).resolve().parent / "golden"


def _bits_equal(a: QSpace, b: QSpace):
    assert a.nblk == b.nblk and a.info.get("itags") == b.info.get("itags")
    for x, y in zip(a.data, b.data):
        assert np.asarray(x).tobytes(order="F") == np.asarray(y).tobytes(order="F")


def test_container_round_trip_through_device(ctx):
    z = np.load(G / "contract_golden.npz")
    cases = json.loads(str(z["cases"]))
    for c in cases[:12]:
        A = QSpace.from_dict(unpack(f"{c['name']}_A", z))
        wa = to_wire(A)
        T = upload_wire(wa, ctx)
        assert np.array_equal(T.to_wire(), wa)       # byte-identical container back
        T.free()


@pytest.mark.parametrize("prec,tol", [("fp64", 1e-14), ("split", 1e-12)])
def test_contractions_from_containers(ctx, prec, tol):
    z = np.load(G / "contract_golden.npz")
    for c in json.loads(str(z["cases"])):
        n = c["name"]
        A, B, R = unpack(f"{n}_A", z), unpack(f"{n}_B", z), unpack(f"{n}_C", z)
        qa, qb = QSpace.from_dict(A), QSpace.from_dict(B)
        TA, TB = upload_wire(to_wire(qa), ctx), upload_wire(to_wire(qb), ctx)
        TC = contract_dev(TA, c["ia"], TB, c["ib"], c["perm"], prec=prec)
        C = from_wire(TC.to_wire())
        assert_qspace_close(C, R, tol)
        assert C.info.get("itags") == R["info"].get("itags"), n
        if prec == "fp64":
            _bits_equal(C, contractQS(qa, c["ia"], qb, c["ib"], c["perm"], prec=prec, ctx=ctx))
        for t in (TA, TB, TC):
            t.free()
