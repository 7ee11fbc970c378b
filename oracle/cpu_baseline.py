"""Timed CPU baseline of the grouped block products -- the reference's own
algorithm restated (checker/baseline only, never part of the product).

QSpace computes every block pair with one BLAS call (zgemm/dgemm through
wbarray::contract, Source/wbarray.cc:3389-3500 and Source/wbarray_blas.cc:
121-213) inside an OpenMP loop over output blocks (Source/QSpace.cc:
4363-4393) -- the recommended exclusive threading is QSP_NUM_THREADS = cores,
OMP_NUM_THREADS = 1 (Docu/README-v3.txt:135-160).  This module does the
same: a thread pool of ``cores`` workers over the pairs, each pair one
single-threaded OpenBLAS GEMM (numpy's bundled OpenBLAS, ILP64).

Run as a module so that OPENBLAS_NUM_THREADS=1 is set before numpy loads:
    python -m oracle.cpu_baseline --npairs 2000 --seed 0 --steps 3
prints one JSON line with the FP64-equivalent TFLOP/s.
"""
from __future__ import annotations

import os

os.environ.setdefault("OPENBLAS_NUM_THREADS", "1")
os.environ.setdefault("OMP_NUM_THREADS", "1")

import argparse  # noqa: E402
import concurrent.futures as cf  # noqa: E402
import json  # noqa: E402
import sys  # noqa: E402
import time  # noqa: E402

import numpy as np  # noqa: E402


def grouped_products(A, B, afac, threads: int):
    """C_p = afac_p * A_p @ B_p for all pairs, `threads` pairs at a time."""
    out = [None] * len(A)

    def one(p):
        out[p] = afac[p] * (A[p] @ B[p])

    order = sorted(range(len(A)), key=lambda p: -A[p].shape[0] * A[p].shape[1] * B[p].shape[1])
    with cf.ThreadPoolExecutor(max_workers=threads) as ex:
        list(ex.map(one, order))
    return out


def block_eigs(blocks, threads: int):
    """numpy eigh (LAPACK dsyevd) of every block, `threads` blocks at a time:
    the OpenMP loop of QSpace::EigenSymmetric (Source/QSpace.cc:4789-4811)
    calling wbEigenS -> dsyevd (Source/wbarray_blas.cc:501-660)."""
    out = [None] * len(blocks)

    def one(i):
        out[i] = np.linalg.eigh(blocks[i])

    order = sorted(range(len(blocks)), key=lambda i: -blocks[i].shape[0])
    with cf.ThreadPoolExecutor(max_workers=threads) as ex:
        list(ex.map(one, order))
    return out


def main_eig(a):
    root = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
    sys.path.insert(0, root)
    from qspace_gb300.workloads import nrg_eig_blocks
    blocks = nrg_eig_blocks(a.seed)
    flops = float(sum(10.0 / 3.0 * b.shape[0] ** 3 for b in blocks))
    block_eigs(blocks, a.threads)
    ts = []
    t_all = time.perf_counter()
    for _ in range(a.steps):
        t0 = time.perf_counter()
        block_eigs(blocks, a.threads)
        ts.append(time.perf_counter() - t0)
        if time.perf_counter() - t_all > a.max_seconds:
            break
    t = float(np.median(ts))
    print(json.dumps({"value": flops / t / 1e12, "unit": "TFLOP/s", "cores": a.threads, "seconds_per_step": t,
                      "steps": len(ts), "flops": flops,
                      "sample": f"all {len(blocks)} blocks ({sum(b.shape[0] for b in blocks)} states) per step"}))


def main_nrg(a):
    """Wilson-chain NRG iterations (the same step and parameters as the
    bench's device row: Nkeep 4096, Lambda 2.5, eps -0.2, U 0.6, t 1,
    deps 1e-8) with the oracle backend: numpy block operations and LAPACK
    eigh through OpenBLAS on all host cores.  Reports the median of the last
    three of ten iterations (the kept space is full from the seventh on)."""
    root = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
    sys.path.insert(0, root)
    from oracle.nrg_port import OracleBackend
    from qspace_gb300.nrg import initial_space, step
    be = OracleBackend()
    K = initial_space(be, -0.2, 0.6)
    ts = []
    t_all = time.perf_counter()
    for _ in range(10):
        t0 = time.perf_counter()
        K = step(K, be, 1.0, 2.5, nkeep=4096, deps=1e-8)
        ts.append(time.perf_counter() - t0)
        if time.perf_counter() - t_all > a.max_seconds:
            break
    t = float(np.median(ts[-3:]))
    print(json.dumps({"unit": "ms", "cores": a.threads, "seconds_per_step": t, "steps": len(ts),
                      "sample": f"{len(ts)} iterations, median of the last 3 ({K.nkept} kept, {K.ntotal} product states)"}))


def main(argv=None):
    ap = argparse.ArgumentParser()
    ap.add_argument("--npairs", type=int, default=2000)
    ap.add_argument("--seed", type=int, default=0)
    ap.add_argument("--steps", type=int, default=3)
    ap.add_argument("--warmup", type=int, default=1)
    ap.add_argument("--threads", type=int, default=os.cpu_count() or 1)
    ap.add_argument("--max-seconds", type=float, default=60.0)
    ap.add_argument("--eig", action="store_true", help="block eigendecompositions instead of block products")
    ap.add_argument("--nrg", action="store_true", help="Wilson-chain NRG iterations instead of block products")
    a = ap.parse_args(argv)
    if a.eig:
        return main_eig(a)
    if a.nrg:
        return main_nrg(a)
    root = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
    sys.path.insert(0, root)
    from qspace_gb300.workloads import grouped_pairs
    w = grouped_pairs(seed=a.seed, npairs=a.npairs, complex_data=True)
    flops = float(np.sum(8.0 * w["M"].astype(float) * w["N"] * w["K"]))
    for _ in range(a.warmup):
        grouped_products(w["A"], w["B"], w["afac"], a.threads)
    ts = []
    t_all = time.perf_counter()
    for _ in range(a.steps):
        t0 = time.perf_counter()
        grouped_products(w["A"], w["B"], w["afac"], a.threads)
        ts.append(time.perf_counter() - t0)
        if time.perf_counter() - t_all > a.max_seconds:
            break
    t = float(np.median(ts))
    print(json.dumps({"value": flops / t / 1e12, "unit": "TFLOP/s", "cores": a.threads,
                      "seconds_per_step": t, "steps": len(ts), "flops": flops,
                      "sample": f"all {a.npairs} pairs of the workload per step"}))


if __name__ == "__main__":
    main()
