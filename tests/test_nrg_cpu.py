"""The NRG iteration driver (qspace_gb300.nrg.step) run on the CPU with the
oracle backend: without truncation its spectrum after L sites is the exact
spectrum of the dense Wilson chain (Kronecker products with Jordan-Wigner
signs); with truncation every iteration keeps the markSet selection; and
three truncated chains (31 iterations, up to 2076 states) reproduce the
fixture made by running the same iteration on the reference's own
contractQS / permuteQS / plusQS / eigQS (tests/golden/make_nrg_golden.py)."""
import numpy as np

from oracle.nrg_port import OracleBackend, dense_chain
from qspace_gb300.nrg import initial_space, step


def _spectrum(K):
    return np.sort(np.concatenate([e for e in K.E.values()]))


def test_untruncated_chain_matches_exact_diagonalisation():
    be = OracleBackend()
    Lam, eps, U = 2.5, -0.3, 0.8
    ts = [1.0, 0.7, 0.55, 0.4]
    K = initial_space(be, eps, U)
    for N, t in enumerate(ts):
        K = step(K, be, t, Lam, nkeep=-1)
        ref = dense_chain(N + 2, eps, U, ts, Lam)
        got = _spectrum(K)
        assert got.shape == ref.shape == (4 ** (N + 2),)
        assert np.max(np.abs(got - ref)) <= 1e-12 * max(1.0, np.abs(ref).max())


def test_truncated_iterations_keep_the_lowest_states():
    be = OracleBackend()
    K = initial_space(be, 0.1, 0.5)
    for t in (1.0, 0.8, 0.6, 0.5, 0.4):
        prev = K.nkept
        K = step(K, be, t, 2.0, nkeep=60)
        kept = _spectrum(K)
        assert K.ntotal == 4 * prev
        assert K.nkept == min(60, K.ntotal) == len(kept)
        assert np.array_equal(kept, K.Eall[:K.nkept])     # markSet with deps = 0: the lowest states


def _golden():
    import json
    from pathlib import Path
    z = np.load(Path(__file__).resolve().parent / "golden" / "nrg_golden.npz")
    return z, json.loads(str(z["runs"]))


def chain_matches_reference(backend_of, tol):
    """Runs every chain of the reference fixture (tests/golden/make_nrg_golden.py:
    the same iteration on the reference's own contractQS / permuteQS / plusQS /
    eigQS) with the given backend; per iteration the same states before and
    after the truncation, the same kept states in every sector and the same
    levels (relative to the largest |E|)."""
    from qspace_gb300.nrg import wilson_hopping
    z, runs = _golden()
    assert len(runs) == 3
    for r in runs:
        be = backend_of()
        K = initial_space(be, r["eps"], r["U"])
        for n in range(r["iters"]):
            K = step(K, be, wilson_hopping(n, r["Lambda"], r["z"]), r["Lambda"], nkeep=r["nkeep"], deps=r["deps"])
            key = f"{r['name']}_{n}"
            assert (K.nkept, K.ntotal) == tuple(z[key + "_sizes"]), key
            labs = sorted(K.E)
            assert np.array_equal(np.array(labs, np.int32).reshape(len(labs), -1), z[key + "_labels"]), key
            assert np.array_equal([len(K.E[l]) for l in labs], z[key + "_kept"]), key
            ref = z[key + "_E"]
            assert np.max(np.abs(K.Eall - ref)) <= tol * np.abs(ref).max(), key


def test_oracle_chain_matches_reference_fixture():
    chain_matches_reference(OracleBackend, 1e-12)


def test_product_basis_packed_construction():
    """The packed product basis A4 / A4Z and the diagonal product term, built
    with whole-array operations, equal the block-by-block construction:
    identity slices of each (kept sector, site state) inside its combined
    sector, the fermionic sign on A4Z, E_K on the diagonal."""
    from qspace_gb300 import nrg
    rng = np.random.default_rng(7)
    E = {}
    for q in range(-3, 4):
        for s2 in (-1, 1):
            E[(q, s2)] = np.sort(rng.standard_normal(int(rng.integers(1, 6))))
    K = nrg.KeptSpace(5, E)
    A4, A4Z, D, off = nrg._fusion(K)
    Q, Qz = A4.qspace(), A4Z.qspace()
    b = 0
    for s in nrg.SITE_LABELS:
        for qk in sorted(E):
            qn = (qk[0] + s[0], qk[1] + s[1])
            d = len(E[qk])
            blk = np.zeros((d, 1, D[qn]))
            blk[:, 0, off[(qk, s)]:off[(qk, s)] + d] = np.eye(d)
            assert tuple(Q.Q[0][b]) == qk and tuple(Q.Q[1][b]) == s and tuple(Q.Q[2][b]) == qn
            assert np.array_equal(Q.data[b], blk)
            assert np.array_equal(Qz.data[b], nrg.parity(qk, K.nsites) * blk)
            b += 1
    H = nrg._diag_product(K, D, off, 1.5).qspace()
    diag = {qn: np.zeros(dd) for qn, dd in D.items()}
    for (qk, s), o in off.items():
        qn = (qk[0] + s[0], qk[1] + s[1])
        diag[qn][o:o + len(E[qk])] = 1.5 * E[qk]
    for i, lab in enumerate(sorted(diag)):
        assert tuple(H.Q[0][i]) == lab and tuple(H.Q[1][i]) == lab
        assert np.array_equal(H.data[i], np.diag(diag[lab]))
