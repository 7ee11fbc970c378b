"""Block eig / SVD / Gram-Schmidt on the GPU (FP64) vs numpy and the oracle;
eigQS-style truncation vs the oracle's markSet restatement."""
import numpy as np
import pytest

from oracle import qs_oracle as orc
from qspace_gb300 import QSpace
from qspace_gb300.linalg import eigQS, eig_blocks, gs_reortho, svd_blocks

pytestmark = pytest.mark.gpu


def _sym(rng, n, cplx=False):
    a = rng.standard_normal((n, n))
    if cplx:
        a = a + 1j * rng.standard_normal((n, n))
    return (a + a.conj().T) / 2


@pytest.mark.parametrize("cplx", [False, True])
def test_eig_blocks_uneven_sizes(ctx, cplx):
    rng = np.random.default_rng(3)
    sizes = [1, 2, 5, 17, 32, 32, 33, 64, 150, 3, 700 if not cplx else 200]
    blocks = [_sym(rng, n, cplx) for n in sizes]
    Es, Us = eig_blocks(blocks, ctx)
    for H, E, U in zip(blocks, Es, Us):
        ref = np.linalg.eigvalsh(H)
        scale = max(1.0, np.abs(ref).max())
        assert np.max(np.abs(E - ref)) <= 1e-12 * scale
        n = H.shape[0]
        assert np.max(np.abs(U.conj().T @ U - np.eye(n))) <= 1e-12 * max(1, n)
        assert np.max(np.abs(H @ U - U * E[None, :])) <= 1e-11 * scale


@pytest.mark.parametrize("cplx", [False, True])
def test_eig_blocks_repeated_sizes(ctx, cplx):
    """Blocks of one size solved together: scattered through the arena (staged
    copies), adjacent (in place), next to blocks of the Jacobi range."""
    rng = np.random.default_rng(8)
    sizes = [40, 7, 40, 90, 40, 90, 16, 16, 17, 17, 120, 120, 120, 5, 40]
    blocks = [_sym(rng, n, cplx) for n in sizes]
    blocks[3] = blocks[3] * 1e-3          # scales differ within a size group
    Es, Us = eig_blocks(blocks, ctx)
    for H, E, U in zip(blocks, Es, Us):
        ref = np.linalg.eigvalsh(H)
        scale = max(1e-3, np.abs(ref).max())
        assert np.max(np.abs(E - ref)) <= 1e-12 * scale
        n = H.shape[0]
        assert np.max(np.abs(U.conj().T @ U - np.eye(n))) <= 1e-12 * max(1, n)
        assert np.max(np.abs(H @ U - U * E[None, :])) <= 1e-11 * scale


def test_eigQS_truncation_matches_oracle(ctx):
    rng = np.random.default_rng(5)
    labels = np.arange(-3, 4, dtype=np.int32).reshape(-1, 1)
    data = [_sym(rng, int(rng.integers(1, 40))) for _ in labels]
    H = QSpace([labels.copy(), labels.copy()], data)
    for nkeep in (-1, 10, 37, 100):
        Etot, I = eigQS(H, Nkeep=nkeep, ctx=ctx)
        ref_E = [np.linalg.eigvalsh(d) for d in data]
        keep, nk = orc.mark_keep(ref_E, nkeep)
        assert I["NK"] == nk
        kept = sum(d.shape[1] for d in I["AK"].data) if I["AK"].nblk else 0
        assert kept == nk
        assert np.allclose(np.sort(np.concatenate(ref_E)), Etot, atol=1e-12 * 10)


def test_svd_blocks(ctx):
    rng = np.random.default_rng(9)
    shapes = [(1, 1), (5, 3), (3, 5), (40, 40), (100, 37), (37, 100), (128, 65)]
    blocks = [rng.standard_normal(s) for s in shapes]
    Us, Ss, Vs = svd_blocks(blocks, ctx)
    for A, U, S, Vt in zip(blocks, Us, Ss, Vs):
        ref = np.linalg.svd(A, compute_uv=False)
        assert np.max(np.abs(np.sort(S)[::-1] - ref)) <= 1e-12 * ref.max()
        assert np.max(np.abs((U * S[None, :]) @ Vt - A)) <= 1e-12 * max(1.0, np.abs(A).max()) * 10
        k = min(A.shape)
        assert np.max(np.abs(U.T @ U - np.eye(k))) <= 1e-12 * k
        assert np.max(np.abs(Vt @ Vt.T - np.eye(k))) <= 1e-12 * k


def test_svd_blocks_complex(ctx):
    rng = np.random.default_rng(10)
    shapes = [(1, 1), (6, 2), (2, 6), (50, 50), (90, 33), (33, 90)]
    blocks = [rng.standard_normal(s) + 1j * rng.standard_normal(s) for s in shapes]
    Us, Ss, Vs = svd_blocks(blocks, ctx)
    for A, U, S, Vt in zip(blocks, Us, Ss, Vs):
        ref = np.linalg.svd(A, compute_uv=False)
        assert np.max(np.abs(np.sort(S)[::-1] - ref)) <= 1e-12 * ref.max()
        assert np.max(np.abs((U * S[None, :]) @ Vt - A)) <= 1e-11 * max(1.0, np.abs(A).max())
        k = min(A.shape)
        assert np.max(np.abs(U.conj().T @ U - np.eye(k))) <= 1e-12 * k
        assert np.max(np.abs(Vt @ Vt.conj().T - np.eye(k))) <= 1e-12 * k


def test_svd_many_small_blocks(ctx):
    """40 000 blocks of one small shape (more than one batched-Jacobi group)
    next to a few large ones (polar-decomposition solver on the lanes)."""
    rng = np.random.default_rng(13)
    blocks = [rng.standard_normal((3, 2)) for _ in range(40000)] + [rng.standard_normal((70, 45)),
                                                                   rng.standard_normal((45, 70))]
    Us, Ss, Vs = svd_blocks(blocks, ctx)
    for i in list(range(0, 40000, 997)) + [39999, 40000, 40001]:
        A, U, S, Vt = blocks[i], Us[i], Ss[i], Vs[i]
        assert np.allclose(S, np.linalg.svd(A, compute_uv=False), rtol=1e-12, atol=1e-13)
        assert np.max(np.abs((U * S[None, :]) @ Vt - A)) <= 1e-12 * max(1.0, np.abs(A).max()) * 10


def test_svd_not_converged_is_an_error(ctx):
    """One Jacobi sweep at a tolerance of 1e-15 cannot diagonalise a dense
    random 120 x 90 block: the call reports QS_ERR_NUMERIC instead of
    returning unconverged factors."""
    from qspace_gb300._capi import QSError
    rng = np.random.default_rng(12)
    blocks = [rng.standard_normal((4, 3)), rng.standard_normal((120, 90))]
    with pytest.raises(QSError, match="did not converge"):
        svd_blocks(blocks, ctx, max_sweeps=1, tol=1e-15)
    # the context stays usable; the default sweep limit converges
    _, Ss, _ = svd_blocks(blocks, ctx)
    assert np.allclose(Ss[1], np.linalg.svd(blocks[1], compute_uv=False), rtol=1e-12, atol=1e-13)


@pytest.mark.parametrize("n,nv", [(1000, 4), (100003, 8), (5, 0), (2_000_000, 3)])
def test_gs_reortho(ctx, n, nv):
    rng = np.random.default_rng(n)
    V = np.linalg.qr(rng.standard_normal((n, nv)))[0] if nv else np.zeros((n, 0))
    v = rng.standard_normal(n)
    got, nrm = gs_reortho(V, v, ctx)
    ref, nref = orc.gs_reortho(V, v)
    assert abs(nrm - nref) <= 1e-12 * nref
    assert np.max(np.abs(got - ref)) <= 1e-12
    if nv:
        assert np.max(np.abs(V.T @ got)) <= 1e-13
