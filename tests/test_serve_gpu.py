"""Serving loop: every result is the same alone and in the mix (bit
identical: deterministic kernels); admission by HBM footprint; host-side
failure injection (bad request, refused admission, cancellation)."""
import numpy as np
import pytest

from qspace_gb300 import contract_dev, upload
from qspace_gb300._capi import QSError
from qspace_gb300.serve import Server
from qspace_gb300.workloads import mps_site_tensor

pytestmark = pytest.mark.gpu


def _same(a, b):
    A, B = a.download(), b.download()
    assert A.nblk == B.nblk
    for qa, qb in zip(A.Q, B.Q):
        assert np.array_equal(qa, qb)
    for x, y in zip(A.data, B.data):
        assert np.array_equal(np.asarray(x), np.asarray(y))


def test_results_identical_alone_and_in_the_mix(ctx):
    tensors = [upload(mps_site_tensor(s), ctx) for s in range(6)]
    jobs = []
    for i, t in enumerate(tensors):
        for prec in ("fp64", "split"):
            jobs.append((t, "12*", t, "12", prec))
    alone = [contract_dev(a, ia, b, ib, prec=p) for (a, ia, b, ib, p) in jobs]
    with Server(nslots=4, hbm_budget=1 << 30, ctx=ctx) as srv:
        tickets = [srv.submit(a, ia, b, ib, prec=p) for (a, ia, b, ib, p) in jobs * 3]
        lat = []
        for k, t in enumerate(tickets):
            T, ms = srv.wait(t)
            lat.append(ms)
            _same(T, alone[k % len(jobs)])
        assert len(lat) == len(tickets) and min(lat) > 0


def test_admission_refused_and_bad_request(ctx):
    A = upload(mps_site_tensor(0), ctx)
    with Server(nslots=2, hbm_budget=1024, ctx=ctx) as srv:
        with pytest.raises(QSError) as e:
            srv.submit(A, "12*", A, "12")
        assert e.value.code == 5  # QS_ERR_OOM: admission refused
    with Server(nslots=2, hbm_budget=1 << 30, ctx=ctx) as srv:
        with pytest.raises(QSError) as e:
            srv.submit(A, "1,1", A, "12")
        assert e.value.code == 1
        # matching sectors whose contracted dims differ: refused when the
        # request is planned
        from qspace_gb300 import QSpace
        q = np.array([[0]], np.int32)
        X = upload(QSpace([q, q.copy()], [np.ones((2, 3))]), ctx)
        Y = upload(QSpace([q, q.copy()], [np.ones((4, 3))]), ctx)
        with pytest.raises(QSError) as e:
            srv.submit(X, "1", Y, "1")
        assert e.value.code == 2


def test_cancel_queued_request(ctx):
    A = upload(mps_site_tensor(4), ctx)
    with Server(nslots=1, hbm_budget=1 << 30, ctx=ctx) as srv:
        tickets = [srv.submit(A, "12*", A, "12", prec="split") for _ in range(40)]
        srv.cancel(tickets[-1])
        with pytest.raises(QSError) as e:
            srv.wait(tickets[-1])
        assert e.value.code == 9
        for t in tickets[:-1]:
            srv.wait(t)


def _projectors(T):
    X = T.download()
    return {tuple(np.asarray(X.Q[0][i]).ravel()): np.asarray(d) @ np.asarray(d).conj().T
            for i, d in enumerate(X.data)}


def test_eig_and_contraction_requests_same_alone_and_in_the_mix(ctx):
    """Block-eig requests (qs_server_submit_eig) mixed with contraction
    requests on four slots: the same kept states, NK, eigenvalues and kept
    eigenspaces as eigQS of the same tensors run alone, and bit-identical
    contraction results."""
    from qspace_gb300.linalg import eigQS_dev
    tensors = [upload(mps_site_tensor(s), ctx) for s in range(4)]
    Hs = [contract_dev(t, "12*", t, "12") for t in tensors]
    alone_c = [contract_dev(t, "12*", t, "12", prec="split") for t in tensors]
    alone_e = [eigQS_dev(H, Nkeep=100, deps=1e-10)[1] for H in Hs]
    with Server(nslots=4, hbm_budget=4 << 30, ctx=ctx) as srv:
        tickets = []
        for _ in range(3):
            for i, t in enumerate(tensors):
                tickets.append(("c", i, srv.submit(t, "12*", t, "12", prec="split")))
                tickets.append(("e", i, srv.submit_eig(Hs[i], 100, 0.0, 1e-10)))
        for kind, i, t in tickets:
            if kind == "c":
                T, _ = srv.wait(t)
                _same(T, alone_c[i])
                continue
            r = srv.wait_eig(t)
            I = alone_e[i]
            assert r["NK"] == I["NK"]
            assert np.array_equal(r["keep"], I["keep"])
            assert np.max(np.abs(r["E"] - I["E"])) <= 1e-12 * max(1.0, np.abs(I["E"]).max())
            P, R = _projectors(r["AK"]), _projectors(I["AK"])
            assert sorted(P) == sorted(R)
            for lab in R:
                assert np.max(np.abs(P[lab] - R[lab])) <= 1e-10


def test_eig_request_errors(ctx):
    A = upload(mps_site_tensor(0), ctx)
    with Server(nslots=1, hbm_budget=1 << 30, ctx=ctx) as srv:
        with pytest.raises(QSError) as e:
            srv.submit_eig(A, 10)             # rank 3: refused at submit
        assert e.value.code == 2
        t = srv.submit(A, "12*", A, "12")
        with pytest.raises(QSError) as e:
            _poll_eig_raw(srv, t)             # a contraction ticket is not an eig request
        assert e.value.code == 1
        srv.wait(t)


def _poll_eig_raw(srv, t):
    import ctypes as C
    from qspace_gb300._capi import check
    done = C.c_int32()
    check(srv.ctx.lib.qs_server_poll_eig(srv.h, t, 0, C.byref(done), None, None, None, None, None, None, None))
