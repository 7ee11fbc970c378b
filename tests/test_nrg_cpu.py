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
