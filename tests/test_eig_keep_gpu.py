"""markSet on the device (qs_mark_keep_dev): the stable order from merging
the blocks' ascending runs, the degeneracy averaging and the cut give the
same keep flags, NK and Etrunc as the host restatement (qs_mark_keep) -- on
the fixtures made by the reference's own eigQS and on random spectra with
exact and near degeneracies, ties across blocks, Nkeep / Etrunc / deps
combinations and the edge cases (empty blocks, Nkeep 0, keep all)."""
import json
from pathlib import Path

import numpy as np
import pytest

from qspace_gb300.linalg import mark_keep, mark_keep_dev
from tests.golden.golden_io import unpack

pytestmark = pytest.mark.gpu

G = Path(__file__).resolve().parent / "golden"


def _same(E, args, ctx):
    kh, nh, eh = mark_keep(E, *args)
    kd, nd, ed = mark_keep_dev(E, *args, ctx=ctx)
    assert nd == nh, (args, nd, nh)
    assert ed == eh, (args, ed, eh)
    for a, b in zip(kd, kh):
        assert np.array_equal(a, b), args
    return kh, nh


def test_reference_fixtures(ctx):
    z = np.load(G / "eig_golden.npz")
    cases = json.loads(str(z["cases"]))
    for c in cases:
        H = unpack(f"{c['name']}_H", z)
        E = [np.linalg.eigvalsh(np.asarray(d)) for d in H["data"]]
        o = c["opts"]
        _, nk = _same(E, (int(o.get("Nkeep", -1)), float(o.get("Etrunc", 0.0)), float(o.get("deps", 0.0))), ctx)
        assert nk == c["NK"], c


@pytest.mark.parametrize("seed", range(6))
def test_random_spectra(ctx, seed):
    rng = np.random.default_rng(seed)
    nb = int(rng.integers(1, 300))
    E = []
    for _ in range(nb):
        k = int(rng.integers(0, 60))
        e = rng.standard_normal(k)
        if seed % 2:
            e = np.round(e, 2)                        # exact ties within and across blocks
        if seed % 3 == 0 and k:
            e[: k // 2] += 1e-11 * rng.standard_normal(k // 2)   # near degeneracies
        E.append(np.sort(e))
    N = sum(len(e) for e in E)
    for nkeep in (-1, 0, 1, N // 3, N // 2, N, N + 5):
        for etrunc in (0.0, 0.5, 2.0):
            for deps in (0.0, 1e-9, 1e-4):
                _same(E, (nkeep, etrunc, deps), ctx)


def test_large_spectrum(ctx):
    """40 000 levels in 336 blocks (the NRG-step size)."""
    rng = np.random.default_rng(9)
    sizes = rng.integers(1, 240, size=336)
    E = [np.sort(np.round(rng.standard_normal(int(k)) * 3, 4)) for k in sizes]
    for args in ((4096, 0.0, 1e-8), (4096, 0.0, 0.0), (8000, 1.0, 0.0), (2000, 0.0, 1e-6)):
        _same(E, args, ctx)


@pytest.mark.parametrize("seed", range(3))
def test_blocks_out_of_order(ctx, seed):
    """Levels of a block need not come ascending: degenerate levels a unit in
    the last place apart in either order (as solvers return them) and blocks
    in arbitrary order give the same flags as the host's stable sort."""
    rng = np.random.default_rng(100 + seed)
    E = []
    for _ in range(int(rng.integers(2, 120))):
        k = int(rng.integers(0, 80))
        e = np.sort(np.round(rng.standard_normal(k) * 1e7, 0))
        for i in range(1, k):                      # swap neighbours a rounding apart
            if rng.random() < 0.3:
                e[i] = np.nextafter(e[i - 1], -np.inf)
        if seed == 2:
            rng.shuffle(e)                          # any order at all
        E.append(e)
    N = sum(len(e) for e in E)
    for nkeep in (1, N // 3, N // 2, N - 1):
        for deps in (0.0, 1e-12, 1e-6):
            _same(E, (nkeep, 0.0, deps), ctx)
