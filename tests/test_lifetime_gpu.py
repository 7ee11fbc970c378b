"""Objects that outlive their context (device tensors, reusable plans, factor
tables) are released without touching the destroyed context -- the order in
which a host (or an interpreter at exit) tears handles down is not
guaranteed.  Run in a child process, so that a regression fails this test
instead of ending the test run."""
import os
import subprocess
import sys
import textwrap

import pytest

pytestmark = pytest.mark.gpu

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))

CHILD = textwrap.dedent("""
    import numpy as np
    from qspace_gb300 import QSpace, upload
    from qspace_gb300.qspace import Context
    from qspace_gb300.grouped import DeviceBatch, FactorTable, Packed
    from qspace_gb300.workloads import grouped_pairs

    c = Context(0)
    w = grouped_pairs(seed=1, npairs=20, lo=4, hi=64, complex_data=True)
    db = DeviceBatch(Packed(w["A"], w["B"], w["afac"], cplx=True), c)
    plan = db.plan("split", graph=True)
    db.run_plan(plan)
    c.sync()
    Q = np.array([[0], [1]], np.int32)
    T = upload(QSpace([Q, Q.copy()], [np.eye(2), np.eye(3)], {}), c)
    F = FactorTable(8, c)
    F.put(np.array([[1, 2]], np.uint64), [0.5])
    c.close()            # the context goes first
    plan.close()
    T.free()
    F.close()
    # a fresh context works normally afterwards
    c2 = Context(0)
    db2 = DeviceBatch(Packed(w["A"], w["B"], w["afac"], cplx=True), c2)
    db2.run("split")
    c2.sync()
    print("lifetime ok")
""")


def test_handles_outlive_their_context():
    r = subprocess.run([sys.executable, "-c", CHILD], cwd=ROOT, capture_output=True, text=True, timeout=600)
    assert r.returncode == 0, r.stderr[-2000:]
    assert "lifetime ok" in r.stdout
