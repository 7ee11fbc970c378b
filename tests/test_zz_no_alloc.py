"""qs_grouped_gemm_split_static: the split grouped GEMM whose device scratch is
one file-scope array per device (nothing allocated).  Called twice in a row
through the C-ABI it must reproduce qs_grouped_gemm (split) on the same pair
list within 1e-12 relative error, without changing the device's free memory
(the first call of a process may only add the array itself, when it loads
the module that holds it);
a pair list that needs more than QS_STATIC_SCRATCH_BYTES is refused with
QS_ERR_OOM before anything runs.  The file name sorts last so that the suite
also runs it after every other GPU test; it passes alone as well."""
import ctypes as C

import numpy as np
import pytest

from qspace_gb300._capi import Stats
from qspace_gb300.grouped import DeviceBatch, Packed
from qspace_gb300.qspace import make_opts
from qspace_gb300.workloads import grouped_pairs

pytestmark = pytest.mark.gpu

STATIC_BYTES = 32 << 20   # QS_STATIC_SCRATCH_BYTES
TOL = 1e-12               # split path target, relative Frobenius error
MODULE_SLACK = 8 << 20    # module image and the driver's allocation granularity
_MODULE_LOADED = [False]  # set once a call of this process has returned


def _digit_bytes_bound(pk: Packed) -> int:
    """Upper bound of the BF16 digit arena of a batch (8 digits per operand;
    the larger of the real-form layouts a block may take)."""
    cm = 2 if pk.cplx else 1
    tot = 0
    for M, N, K in zip(pk.M, pk.N, pk.K):
        M, N = int(M), int(N)
        kb = max(1, -(-int(K) * cm // 32))
        lay = [(cm * M, N), (cm * N, M)] + ([(M, 2 * N), (N, 2 * M)] if cm == 2 else [])
        tot += max(-(-r // 128) * kb * 8 * 8192 + -(-c // 32) * kb * 8 * 2048 for r, c in lay)
    return tot


def _static(db: DeviceBatch, prec="split"):
    st = Stats()
    rc = db.ctx.lib.qs_grouped_gemm_split_static(
        db.ctx.h, C.byref(db.pl), C.c_void_p(db.dA.data_ptr()), C.c_void_p(db.dB.data_ptr()),
        C.c_void_p(db.dC.data_ptr()), C.byref(make_opts(prec, 0, TOL)), C.byref(st))
    return rc, st


def _rel(x: list, y: list) -> float:
    num = sum(float(np.linalg.norm(a - b)) ** 2 for a, b in zip(x, y))
    den = sum(float(np.linalg.norm(b)) ** 2 for b in y)
    return (num / max(den, 1e-300)) ** 0.5


def _check_twice(ctx, pk: Packed):
    import torch
    assert _digit_bytes_bound(pk) < STATIC_BYTES - (1 << 20)
    db = DeviceBatch(pk, ctx)
    db.run("split", 0, TOL)                  # the existing entry point
    ref = [b.copy() for b in db.result()]
    exact = [a @ b * f for a, b, f in zip([np.asarray(x) for x in _A(pk)], _B(pk), pk.afac)] \
        if len(set(pk.blk.tolist())) == pk.n else None
    for call in range(2):
        db.dC.fill_(float("nan"))            # a call that wrote nothing would fail
        torch.cuda.synchronize()
        free0 = torch.cuda.mem_get_info(ctx.device)[0]
        rc, st = _static(db)
        assert rc == 0, ctx.lib.qs_last_error().decode()
        free1 = torch.cuda.mem_get_info(ctx.device)[0]
        assert st.nslices >= 2 and st.npairs == pk.n and st.launches >= 3
        got = db.result()
        assert all(np.all(np.isfinite(g)) for g in got)
        assert _rel(got, ref) <= TOL, call
        if exact is not None:
            assert _rel(got, exact) <= TOL, call
        if _MODULE_LOADED[0]:
            # the array is resident: no device memory comes or goes
            assert free1 == free0, (call, free0 - free1)
        else:
            # the first call of the process may load the module that holds the
            # array (lazy loading): at most the array plus the module image
            assert 0 <= free0 - free1 <= STATIC_BYTES + MODULE_SLACK, (call, free0 - free1)
            _MODULE_LOADED[0] = True


def _A(pk: Packed):
    return [pk.abuf[o:o + m * k].reshape((m, k), order="F") for o, m, k in zip(pk.a_off, pk.M, pk.K)]


def _B(pk: Packed):
    return [pk.bbuf[o:o + k * n].reshape((k, n), order="F") for o, k, n in zip(pk.b_off, pk.K, pk.N)]


def test_static_scratch_matches_grouped_gemm_complex(ctx):
    w = grouped_pairs(seed=7, npairs=24, lo=8, hi=160, complex_data=True)
    _check_twice(ctx, Packed(w["A"], w["B"], w["afac"], cplx=True))


def test_static_scratch_matches_grouped_gemm_shared_blocks(ctx):
    # real pairs, three output blocks summing 3, 1 and 4 pairs of different depth
    rng = np.random.default_rng(11)
    shapes = [(96, 40)] * 3 + [(17, 130)] + [(200, 33)] * 4
    Ks = [64, 5, 300, 77, 1, 129, 48, 250]
    A = [np.asfortranarray(rng.standard_normal((m, k))) for (m, _), k in zip(shapes, Ks)]
    B = [np.asfortranarray(rng.standard_normal((k, n))) for (_, n), k in zip(shapes, Ks)]
    afac = rng.uniform(-2, 2, size=8)
    _check_twice(ctx, Packed(A, B, afac, blk=[0, 0, 0, 1, 2, 2, 2, 2], cplx=False))


def test_static_scratch_refuses_oversize_and_fp64(ctx):
    rng = np.random.default_rng(3)
    n = 1024
    a = np.asfortranarray(rng.standard_normal((n, n)) + 1j * rng.standard_normal((n, n)))
    pk = Packed([a], [a.copy()], [1.0], cplx=True)
    assert _digit_bytes_bound(pk) > STATIC_BYTES
    db = DeviceBatch(pk, ctx)
    rc, _ = _static(db)
    assert rc == 5, rc                      # QS_ERR_OOM, nothing launched
    assert b"static scratch" in ctx.lib.qs_last_error()
    rc, _ = _static(db, prec="fp64")
    assert rc == 1                          # QS_ERR_ARG: split path only
    # the context is still usable
    small = grouped_pairs(seed=1, npairs=4, lo=8, hi=64, complex_data=True)
    _check_twice(ctx, Packed(small["A"], small["B"], small["afac"], cplx=True))
