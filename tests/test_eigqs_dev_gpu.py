"""eigQS on a device-resident QSpace (qs_eigQS_dev): the same eigenvectors
and truncation as the host-side eigQS (bit for bit: same kernels on the same
blocks), the oracle's markSet restatement for the kept set (Nkeep, Etrunc and
degeneracy averaging), kept states = the lowest of each block, and AK, AD
orthonormal with AK^H H AK diagonal."""
import numpy as np
import pytest

from oracle import qs_oracle as orc
from qspace_gb300 import QSpace, upload
from qspace_gb300.linalg import eigQS, eigQS_dev

pytestmark = pytest.mark.gpu


def _herm(rng, n, cplx):
    a = rng.standard_normal((n, n))
    if cplx:
        a = a + 1j * rng.standard_normal((n, n))
    return (a + a.conj().T) / 2


def _H(seed, cplx, sizes):
    rng = np.random.default_rng(seed)
    labels = np.array([[q, s] for q, s in zip(range(-len(sizes) // 2, len(sizes)), [1, -1] * len(sizes))][:len(sizes)],
                      np.int32)
    data = [_herm(rng, n, cplx) for n in sizes]
    return QSpace([labels.copy(), labels.copy()], data, {"itags": ["K", "K*"]})


def _blocks(Q: QSpace):
    return {tuple(np.asarray(Q.Q[0][i]).ravel()): np.asarray(d) for i, d in enumerate(Q.data)}


@pytest.mark.parametrize("cplx", [False, True])
@pytest.mark.parametrize("nkeep,etrunc,deps", [(-1, 0.0, 0.0), (25, 0.0, 0.0), (60, 0.0, 1e-3), (200, 1.5, 0.0)])
def test_eigqs_dev_matches_host_and_oracle(ctx, cplx, nkeep, etrunc, deps):
    sizes = [1, 7, 40, 40, 17, 64, 3, 33, 40, 120]
    H = _H(11, cplx, sizes)
    T = upload(H, ctx)
    Etot, I = eigQS_dev(T, Nkeep=nkeep, Etrunc=etrunc, deps=deps)
    Eh, Ih = eigQS(H, Nkeep=nkeep, Etrunc=etrunc, deps=deps, ctx=ctx)
    assert np.array_equal(Etot, Eh) and I["NK"] == Ih["NK"]
    ref_E = [np.linalg.eigvalsh(d) for d in H.data]
    keep_ref, nk_ref = orc.mark_keep(ref_E, nkeep, etrunc, deps)
    assert I["NK"] == nk_ref
    AK, AD = I["AK"].download(), I["AD"].download()
    for part, host in ((AK, Ih["AK"]), (AD, Ih["AD"])):
        a, b = _blocks(part), _blocks(host)
        assert a.keys() == b.keys()
        for k in a:
            assert np.asarray(a[k]).tobytes(order="F") == np.asarray(b[k]).tobytes(order="F")
    # kept = the lowest states of each block; vectors orthonormal, H diagonal
    # on them; the reported levels are the eigenvalues, averaged over
    # degenerate clusters when deps > 0 (as markSet writes them back)
    rep_E = orc.average_levels(ref_E, deps)
    o = 0
    ak, ad = _blocks(AK), _blocks(AD)
    for i, (d, e) in enumerate(zip(H.data, ref_E)):
        key = tuple(np.asarray(H.Q[0][i]).ravel())
        n = d.shape[0]
        flags = I["keep"][o:o + n]
        k = int(flags.sum())
        assert np.all(flags[:k]) and not np.any(flags[k:])
        assert k == int(np.sum(keep_ref[i]))
        U = np.hstack([x for x in (ak.get(key), ad.get(key)) if x is not None])
        assert U.shape == (n, n)
        assert np.max(np.abs(U.conj().T @ U - np.eye(n))) <= 1e-12 * n
        D = U.conj().T @ d @ U
        assert np.max(np.abs(D - np.diag(np.diag(D)))) <= 1e-11 * max(1.0, np.abs(e).max())
        assert np.max(np.abs(np.diag(D).real - e)) <= 1e-11 * max(1.0, np.abs(e).max())
        assert np.max(np.abs(rep_E[i] - I["E"][o:o + n])) <= 1e-11 * max(1.0, np.abs(e).max())
        o += n
    assert AK.info.get("itags") == ["K", "K*"]
    for t in (T, I["AK"], I["AD"]):
        t.free()


def test_eigqs_dev_rejects_off_diagonal(ctx):
    from qspace_gb300._capi import QSError
    H = QSpace([np.array([[0], [1]], np.int32), np.array([[1], [0]], np.int32)], [np.eye(2), np.eye(2)])
    T = upload(H, ctx)
    with pytest.raises(QSError) as e:
        eigQS_dev(T)
    assert e.value.code == 3


@pytest.mark.parametrize("deps", [0.0, 1e-10])
def test_eigqs_dev_degenerate_levels(ctx, deps):
    """Blocks with exactly degenerate multiplets at a large scale (the NRG
    Hamiltonian before rescaling): the solver returns degenerate levels only
    up to rounding, in either order.  Each block's levels come back
    non-decreasing, its kept states are its first columns, and they are
    eigenvectors of their levels."""
    rng = np.random.default_rng(21)
    sizes = [650, 380, 24, 9, 200, 130]
    data = []
    for n in sizes:
        lv = np.round(rng.standard_normal(-(-n // 6)) * 4e7, 3)
        d = np.sort(np.repeat(lv, 6)[:n])           # sextets (one partial)
        Qm, _ = np.linalg.qr(rng.standard_normal((n, n)))
        data.append((Qm * d) @ Qm.T)
    labels = np.arange(len(sizes), dtype=np.int32).reshape(-1, 1)
    H = QSpace([labels.copy(), labels.copy()], [(x + x.T) / 2 for x in data])
    T = upload(H, ctx)
    N = sum(sizes)
    for nkeep in (N // 4, N // 2 + 1, N - 7):
        Etot, I = eigQS_dev(T, Nkeep=nkeep, deps=deps)
        ak = _blocks(I["AK"].download())
        o = 0
        for i, (d, n) in enumerate(zip(H.data, sizes)):
            e = I["E"][o:o + n]
            assert np.all(np.diff(e) >= 0)
            flags = I["keep"][o:o + n]
            k = int(flags.sum())
            assert np.all(flags[:k]) and not np.any(flags[k:])
            if k:
                U = ak[(i,)]
                assert U.shape == (n, k)
                r = d @ U - U * e[None, :k]
                assert np.max(np.abs(r)) <= 1e-9 * np.abs(e).max()
            o += n
        for t in (I["AK"], I["AD"]):
            t.free()
    T.free()


def test_eigqs_reference_fixtures(ctx):
    """eigQS (device-resident and host forms) on the Hamiltonians of the
    reference's own eigQS fixtures: the same NK, kept states per sector and
    levels as the reference -- averaged over near-degenerate clusters when
    deps > 0, as markSet writes them back."""
    import json
    from pathlib import Path
    from tests.golden.golden_io import unpack
    z = np.load(Path(__file__).resolve().parent / "golden" / "eig_golden.npz")
    for c in json.loads(str(z["cases"])):
        Hd = unpack(f"{c['name']}_H", z)
        H = QSpace(Hd["Q"], [np.asarray(d) for d in Hd["data"]], {})
        o = c["opts"]
        kw = dict(Nkeep=int(o.get("Nkeep", -1)), Etrunc=float(o.get("Etrunc", 0.0)), deps=float(o.get("deps", 0.0)))
        ref_tot = np.sort(z[f"{c['name']}_Etot"])
        sc = np.abs(ref_tot).max()
        EK = unpack(f"{c['name']}_EK", z)
        ref_k = {tuple(np.asarray(EK["Q"][0][i]).ravel()): np.sort(np.asarray(d).ravel()) for i, d in enumerate(EK["data"])}
        T = upload(H, ctx)
        Etot, I = eigQS_dev(T, **kw)
        assert I["NK"] == c["NK"], c["name"]
        assert np.max(np.abs(Etot - ref_tot)) <= 1e-12 * sc, c["name"]
        o_ = 0
        got_k = {}
        for i, d in enumerate(H.data):
            n = np.asarray(d).shape[0]
            f = I["keep"][o_:o_ + n]
            if f.any():
                got_k[tuple(np.asarray(H.Q[0][i]).ravel())] = I["E"][o_:o_ + n][f]
            o_ += n
        assert got_k.keys() == ref_k.keys(), c["name"]
        for k in ref_k:
            assert np.allclose(got_k[k], ref_k[k], rtol=0, atol=1e-12 * sc), (c["name"], k)
        Eh, Ih = eigQS(H, ctx=ctx, **kw)
        assert Ih["NK"] == c["NK"] and np.max(np.abs(Eh - ref_tot)) <= 1e-12 * sc, c["name"]
        for t in (T, I["AK"], I["AD"]):
            t.free()
