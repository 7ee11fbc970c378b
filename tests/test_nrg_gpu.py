"""The NRG iteration resident on the GPU (qspace_gb300.nrg.step with the
device backend: contractQS / permuteQS / plusQS / eigQS on device tensors):
the exact spectrum of the dense Wilson chain without truncation, and the same
kept energies as the oracle backend over truncated iterations."""
import numpy as np
import pytest

from oracle.nrg_port import OracleBackend, dense_chain
from qspace_gb300.nrg import DeviceBackend, initial_space, step

pytestmark = pytest.mark.gpu


def _spectrum(K):
    return np.sort(np.concatenate([e for e in K.E.values()]))


@pytest.mark.parametrize("prec,tol", [("fp64", 1e-12), ("split", 1e-11)])
def test_device_chain_matches_exact_diagonalisation(ctx, prec, tol):
    be = DeviceBackend(ctx, prec)
    Lam, eps, U = 2.5, -0.3, 0.8
    ts = [1.0, 0.7, 0.55, 0.4]
    K = initial_space(be, eps, U)
    for N, t in enumerate(ts):
        K = step(K, be, t, Lam)
        ref = dense_chain(N + 2, eps, U, ts, Lam)
        got = _spectrum(K)
        assert got.shape == ref.shape
        assert np.max(np.abs(got - ref)) <= tol * max(1.0, np.abs(ref).max())


def test_device_truncated_iterations_match_oracle(ctx):
    dev, cpu = DeviceBackend(ctx, "fp64"), OracleBackend()
    Kd, Kc = initial_space(dev, 0.1, 0.5), initial_space(cpu, 0.1, 0.5)
    # degeneracy averaging keeps spin multiplets together at the cut, so that
    # rounding differences cannot choose different members of a multiplet
    for t in (1.0, 0.8, 0.6, 0.5, 0.4, 0.3):
        Kd, Kc = step(Kd, dev, t, 2.0, nkeep=150, deps=1e-8), step(Kc, cpu, t, 2.0, nkeep=150, deps=1e-8)
        assert Kd.nkept == Kc.nkept and sorted(Kd.E) == sorted(Kc.E)
        for lab in Kc.E:
            assert np.max(np.abs(Kd.E[lab] - Kc.E[lab])) <= 1e-12 * max(1.0, np.abs(Kc.E[lab]).max())
