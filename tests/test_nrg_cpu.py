"""The NRG iteration driver (qspace_gb300.nrg.step) run on the CPU with the
oracle backend: without truncation its spectrum after L sites is the exact
spectrum of the dense Wilson chain (Kronecker products with Jordan-Wigner
signs); with truncation every iteration keeps the markSet selection."""
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
