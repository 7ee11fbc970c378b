"""svdQS and orthoQS host code against the REFERENCE's own MEX functions
called live (oracle/ref.py) on seeded random abelian tensors: rank 2 to 4,
every mix of leg directions, one or two label components, real and complex,
options drawn at random, some with labels that are not conserved.  Each call
must either fail on both sides or agree in labels, block order, shapes,
itags, |data| (free of the singular vectors' phases), kept count, sfac and
flag.  The block SVDs are LAPACK's (numpy), so this runs without a GPU;
skipped where the reference is not compiled (oracle/_ref)."""
import numpy as np
import pytest

from oracle import ref
from qspace_gb300.linalg import _OrthoPlan, _SvdLayout
from qspace_gb300.qspace import QSpace
from tests.golden.make_svdqs_golden import psi

pytestmark = pytest.mark.skipif(not (ref.available("svdQS") and ref.available("orthoQS")),
                                reason="reference oracle not built here (oracle/_ref)")


def _call_ref(name, A, args_tail, opts, nout):
    lib = ref._fake()
    args = [ref.to_mx(A)] + args_tail
    for k, v in opts.items():
        args += [ref._mx_string(k), ref._arg(v)]
    out = ref.call(name, args, nout)
    info = out[-1]
    f = {k: ref._np_of(lib.mxGetField(info, 0, k.encode())).ravel()[0] for k in ("Nkeep", "sfac", "flag")}
    res = [ref.from_mx(x) for x in out[:-1]]
    for x in out + args:
        lib.mxDestroyArray(x)
    return res, f


def _decomp(mats):
    dec = [np.linalg.svd(M, full_matrices=False) for M in mats]
    return [d[0] for d in dec], [d[1] for d in dec], [d[2] for d in dec]


def _same(R, M):
    r = len(R["Q"])
    assert (R["info"].get("itags") or None) == (M.info.get("itags") or None)
    assert len(R["data"]) == M.nblk
    if not M.nblk:
        return
    assert M.rank == r
    for k in range(r):
        assert np.array_equal(np.asarray(R["Q"][k]).reshape(M.nblk, -1), np.asarray(M.Q[k]).reshape(M.nblk, -1))
    for i in range(M.nblk):
        d = np.asarray(R["data"][i])
        assert (tuple(d.shape) + (1,) * r)[:r] == M.block_dims(i)
        assert np.allclose(np.abs(d).ravel(order="F"), np.abs(np.asarray(M.data[i])).ravel(order="F"),
                           rtol=1e-9, atol=1e-11)


def _random_case(rng, t):
    r = int(rng.integers(2, 5))
    tags = [chr(97 + k) + ("*" if rng.random() < 0.4 else "") for k in range(r)]
    cplx = bool(rng.random() < 0.5)
    A = psi(9000 + t, tags, cplx, int(rng.integers(1, 3)), nb=int(rng.integers(1, 9)))
    if rng.random() < 0.15:       # labels not conserved
        n = len(A["data"])
        for q in A["Q"]:
            q[:] = rng.integers(-1, 2, size=q.shape)
        recs = {tuple(np.concatenate([np.asarray(q[i]).ravel() for q in A["Q"]])) for i in range(n)}
        if len(recs) != n:
            return None
        sec = {}
        for i in range(n):
            shp = [sec.setdefault((k, tuple(np.asarray(A["Q"][k][i]).ravel())), int(rng.integers(1, 4)))
                   for k in range(r)]
            x = rng.standard_normal(shp)
            A["data"][i] = x + 1j * rng.standard_normal(shp) if cplx else x
    opts = {}
    if rng.random() < 0.4:
        opts["Nkeep"] = int(rng.integers(0, 8))
    if rng.random() < 0.3:
        opts["stol"] = float(rng.uniform(0, 2))
    if rng.random() < 0.3:
        opts["Nkmin"] = int(rng.integers(0, 4))
    if rng.random() < 0.3:
        opts["itag"] = ["X", "Y*", "bond"][int(rng.integers(0, 3))]
    return r, A, opts


def _kw(opts):
    return dict(Nkeep=opts.get("Nkeep", -1), Nkmin=opts.get("Nkmin", 0), stol=opts.get("stol"),
                itag=opts.get("itag", ""))


def _compare(run_ref, run_mine):
    try:
        R, f = run_ref()
    except ref.RefError:
        with pytest.raises(ValueError):
            run_mine()
        return False
    *M, info = run_mine()
    for x, m in zip(R, M):
        _same(x, m)
    assert info["Nkeep"] == int(f["Nkeep"]) and info["flag"] == int(f["flag"])
    assert abs(info["sfac"] - float(f["sfac"])) <= 1e-12 * max(1.0, float(f["sfac"]))
    return True


def test_svdqs_random_against_live_reference():
    rng = np.random.default_rng(2024)
    agreed = 0
    for t in range(160):
        c = _random_case(rng, t)
        if c is None:
            continue
        r, A, opts = c
        n = int(rng.integers(1, r))
        idx = [int(x) for x in rng.choice(np.arange(1, r + 1), n, replace=False)]
        K = r - n
        if rng.random() < 0.3:
            opts["permA"] = [int(x) + 1 for x in rng.permutation(K + 1)]
        if rng.random() < 0.3:
            opts["permB"] = [int(x) + 1 for x in rng.permutation(r - K + 1)]

        def mine():
            L = _SvdLayout(QSpace.from_dict(A), idx)
            return L.finish(*_decomp(L.mats), permA=opts.get("permA"), permB=opts.get("permB"), **_kw(opts))

        agreed += _compare(lambda: _call_ref("svdQS", A, [ref._arg(idx)], opts, 4), mine)
    assert agreed >= 60


def test_orthoqs_random_against_live_reference():
    rng = np.random.default_rng(2025)
    agreed = 0
    for t in range(160):
        c = _random_case(rng, t)
        if c is None:
            continue
        r, A, opts = c
        lrdir = [None, ">>", "<<", "LR", "RL", "+", "-"][int(rng.integers(0, 7))]
        n = 1 if lrdir is None else int(rng.integers(1, r))
        idx = [int(x) for x in rng.choice(np.arange(1, r + 1), n, replace=False)]
        if lrdir is not None and rng.random() < 0.3:
            opts["permA"] = [int(x) + 1 for x in rng.permutation(int(rng.integers(2, r + 1)))]
        if lrdir is not None and rng.random() < 0.3:
            opts["permB"] = [int(x) + 1 for x in rng.permutation(int(rng.integers(2, r + 1)))]

        def mine():
            pl = _OrthoPlan(QSpace.from_dict(A), idx, lrdir, opts.get("permA"), opts.get("permB"))
            return pl.finish(*_decomp(pl.L.mats), **_kw(opts))

        tail = [ref._arg(idx)] + ([ref._mx_string(lrdir)] if lrdir else [])
        agreed += _compare(lambda: _call_ref("orthoQS", A, tail, opts, 3), mine)
    assert agreed >= 60
