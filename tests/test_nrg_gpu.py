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


def test_concurrent_runs_through_the_serving_loop_match_runs_alone(ctx):
    """Three NRG runs at different z-shifts drive their contractions and
    eigQS through one serving loop from three host threads at once: every
    run keeps the same states with the same energies as the same run alone
    on the device backend."""
    import threading

    from qspace_gb300.nrg import ServingBackend, kept_schedule, wilson_hopping
    from qspace_gb300.qspace import Context
    from qspace_gb300.serve import Server

    Lam, iters, zs = 2.5, 5, (0.0, 1 / 3, 2 / 3)
    nk = kept_schedule(iters, 60, 200)

    def run(be, z, out):
        K = initial_space(be, -0.2, 0.6)
        for n in range(iters):
            K = step(K, be, wilson_hopping(n, Lam, z), Lam, nkeep=nk[n], deps=1e-8)
        out.append(K)

    alone = []
    for z in zs:
        run(DeviceBackend(ctx, "split"), z, alone)
    mixed = [[] for _ in zs]
    with Server(nslots=4, hbm_budget=8 << 30, ctx=ctx) as srv:
        bes = [ServingBackend(srv, Context(ctx.device), "split") for _ in zs]
        th = [threading.Thread(target=run, args=(be, z, o)) for be, z, o in zip(bes, zs, mixed)]
        for t in th:
            t.start()
        for t in th:
            t.join(300)
        assert all(len(be.latency["eig"]) == iters for be in bes)
    for Ka, (Km,) in zip(alone, mixed):
        assert Km.nkept == Ka.nkept and sorted(Km.E) == sorted(Ka.E)
        for lab in Ka.E:
            assert np.max(np.abs(Km.E[lab] - Ka.E[lab])) <= 1e-12 * max(1.0, np.abs(Ka.E[lab]).max())


@pytest.mark.parametrize("prec,tol", [("fp64", 1e-12), ("split", 1e-11)])
def test_device_chain_matches_reference_fixture(ctx, prec, tol):
    """The device iteration against chains run on the reference's own MEX
    functions (tests/golden/nrg_golden.npz): same truncation in every sector,
    same levels (averaged over degenerate clusters, as eigQS reports them)."""
    from tests.test_nrg_cpu import chain_matches_reference
    chain_matches_reference(lambda: DeviceBackend(ctx, prec), tol)
