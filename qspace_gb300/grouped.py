"""Grouped block products through the C-ABI (qs_grouped_gemm / _host).

A batch is a list of block pairs ``C[blk[p]] (+)= afac[p] * A[p] @ B[p]``;
pairs that share ``blk`` are summed (in order) into one output block -- the
per-output-block loop of contractDATA_group (Source/QSpace_aux.cc:27-355)
with the CG factor ``afac`` of each pair.
"""
from __future__ import annotations

import ctypes as C

import numpy as np

from . import _capi
from ._capi import PairList, Stats, check
from .qspace import Context, default_context, make_opts


class Packed:
    """Flat column-major arenas and the pair list of one batch."""

    def __init__(self, A: list, B: list, afac, blk=None, cplx: bool | None = None):
        n = len(A)
        if cplx is None:
            cplx = any(np.iscomplexobj(x) for x in A) or any(np.iscomplexobj(x) for x in B)
        self.cplx = bool(cplx)
        dt = np.complex128 if cplx else np.float64
        self.M = np.array([a.shape[0] for a in A], np.int32)
        self.K = np.array([a.shape[1] for a in A], np.int32)
        self.N = np.array([b.shape[1] for b in B], np.int32)
        if np.any(np.array([b.shape[0] for b in B]) != self.K):
            raise ValueError("inner dimensions differ")
        blk = np.arange(n, dtype=np.int32) if blk is None else np.asarray(blk, np.int32)
        self.blk = blk
        asz = self.M.astype(np.int64) * self.K
        bsz = self.K.astype(np.int64) * self.N
        self.a_off = np.concatenate([[0], np.cumsum(asz)[:-1]]).astype(np.int64)
        self.b_off = np.concatenate([[0], np.cumsum(bsz)[:-1]]).astype(np.int64)
        # one output block per distinct blk id, in order of first appearance
        self.c_off = np.zeros(n, np.int64)
        self.blocks = []           # (M, N, offset)
        seen = {}
        off = 0
        for p in range(n):
            b = int(blk[p])
            if b not in seen:
                seen[b] = len(self.blocks)
                self.blocks.append((int(self.M[p]), int(self.N[p]), off))
                off += int(self.M[p]) * int(self.N[p])
            self.c_off[p] = self.blocks[seen[b]][2]
        self.c_elems = off
        self.abuf = np.concatenate([np.asarray(a, dt).reshape(-1, order="F") for a in A]) if n else np.zeros(0, dt)
        self.bbuf = np.concatenate([np.asarray(b, dt).reshape(-1, order="F") for b in B]) if n else np.zeros(0, dt)
        self.lda = np.maximum(self.M, 1).astype(np.int32)
        self.ldb = np.maximum(self.K, 1).astype(np.int32)
        self.ldc = np.maximum(self.M, 1).astype(np.int32)
        self.trans = np.zeros(n, np.int32)
        self.afac = np.ascontiguousarray(afac, np.float64)
        self.n = n

    @classmethod
    def from_operands(cls, A: list, B: list, ia, ib, afac, blk=None, cplx: bool | None = None) -> "Packed":
        """A batch whose pairs share operand blocks: pair p multiplies A[ia[p]]
        by B[ib[p]]; each distinct operand block is stored once in the arenas
        (as a contraction's pair list reads its input tensors' blocks)."""
        ia = np.asarray(ia, np.int64)
        ib = np.asarray(ib, np.int64)
        pk = cls([A[i] for i in ia], [B[i] for i in ib], afac, blk=blk, cplx=cplx)
        dt = pk.abuf.dtype
        asz = np.array([a.shape[0] * a.shape[1] for a in A], np.int64)
        bsz = np.array([b.shape[0] * b.shape[1] for b in B], np.int64)
        aoff = np.concatenate([[0], np.cumsum(asz)[:-1]]).astype(np.int64)
        boff = np.concatenate([[0], np.cumsum(bsz)[:-1]]).astype(np.int64)
        pk.abuf = np.concatenate([np.asarray(a, dt).reshape(-1, order="F") for a in A]) if A else np.zeros(0, dt)
        pk.bbuf = np.concatenate([np.asarray(b, dt).reshape(-1, order="F") for b in B]) if B else np.zeros(0, dt)
        pk.a_off = aoff[ia].copy()
        pk.b_off = boff[ib].copy()
        return pk

    def operand_bytes(self) -> int:
        """Bytes of the operand arenas (each stored block once)."""
        return int(self.abuf.nbytes + self.bbuf.nbytes)

    def pair_list(self) -> PairList:
        pl = PairList()
        pl.npairs = self.n
        i32, i64 = _capi.c_int32_p, _capi.c_int64_p
        pl.M, pl.N, pl.K = (x.ctypes.data_as(i32) for x in (self.M, self.N, self.K))
        pl.a_off, pl.b_off, pl.c_off = (x.ctypes.data_as(i64) for x in (self.a_off, self.b_off, self.c_off))
        pl.lda, pl.ldb, pl.ldc = (x.ctypes.data_as(i32) for x in (self.lda, self.ldb, self.ldc))
        pl.trans = self.trans.ctypes.data_as(i32)
        pl.afac = self.afac.ctypes.data_as(_capi.c_double_p)
        pl.c_blk = self.blk.ctypes.data_as(i32)
        pl.is_complex = 1 if self.cplx else 0
        return pl

    def unpack_c(self, cbuf: np.ndarray) -> list:
        return [cbuf[o:o + m * n].reshape((m, n), order="F") for (m, n, o) in self.blocks]

    def flops(self) -> float:
        return float(np.sum((8.0 if self.cplx else 2.0) * self.M.astype(float) * self.N * self.K))


def _dbl(x: np.ndarray):
    return x.view(np.float64).ctypes.data_as(_capi.c_double_p)


def run_packed_host(pk: Packed, prec="fp64", nslices=0, tol=1e-12, ctx: Context | None = None,
                    stats: dict | None = None) -> np.ndarray:
    ctx = ctx or default_context()
    cbuf = np.zeros(pk.c_elems, np.complex128 if pk.cplx else np.float64)
    pl = pk.pair_list()
    o = make_opts(prec, nslices, tol)
    st = Stats()
    check(ctx.lib.qs_grouped_gemm_host(ctx.h, C.byref(pl), _dbl(pk.abuf), len(pk.abuf), _dbl(pk.bbuf),
                                       len(pk.bbuf), _dbl(cbuf), len(cbuf), C.byref(o), C.byref(st)))
    if stats is not None:
        stats.update(st.as_dict())
    return cbuf


class PinnedBatch:
    """Host-side batch in page-locked memory for the end-to-end host API
    (qs_grouped_gemm_host copies in and out inside the call)."""

    def __init__(self, pk: Packed, ctx: Context | None = None):
        import torch
        self.pk = pk
        self.ctx = ctx or default_context()
        self.a = torch.from_numpy(pk.abuf.view(np.float64)).pin_memory()
        self.b = torch.from_numpy(pk.bbuf.view(np.float64)).pin_memory()
        self.c = torch.zeros(pk.c_elems * (2 if pk.cplx else 1), dtype=torch.float64).pin_memory()
        self.pl = pk.pair_list()

    def run(self, prec="split", nslices=0, tol=1e-12, stats: dict | None = None):
        o = make_opts(prec, nslices, tol)
        st = Stats()
        dp = lambda t: C.cast(C.c_void_p(t.data_ptr()), _capi.c_double_p)
        check(self.ctx.lib.qs_grouped_gemm_host(self.ctx.h, C.byref(self.pl), dp(self.a), len(self.pk.abuf),
                                                dp(self.b), len(self.pk.bbuf), dp(self.c), self.pk.c_elems,
                                                C.byref(o), C.byref(st)))
        if stats is not None:
            stats.update(st.as_dict())

    @property
    def h2d_bytes(self) -> int:
        return 8 * (self.a.numel() + self.b.numel())

    @property
    def d2h_bytes(self) -> int:
        return 8 * self.c.numel()


def run_host(w: dict, prec="fp64", nslices=0, tol=1e-12, ctx=None, stats=None) -> list:
    pk = Packed(w["A"], w["B"], w["afac"], cplx=w.get("complex"))
    return pk.unpack_c(run_packed_host(pk, prec, nslices, tol, ctx, stats))


def run_host_blocks(A, B, afac, blk, prec="fp64", nslices=0, tol=1e-12, ctx=None, stats=None) -> list:
    pk = Packed(A, B, afac, blk=blk)
    return pk.unpack_c(run_packed_host(pk, prec, nslices, tol, ctx, stats))


class DeviceBatch:
    """A batch resident in device memory (torch tensors as plain buffers)."""

    def __init__(self, pk: Packed, ctx: Context | None = None):
        import torch
        self.torch = torch
        self.pk = pk
        self.ctx = ctx or default_context()
        dev = torch.device("cuda", self.ctx.device)
        self.dA = torch.from_numpy(pk.abuf.view(np.float64)).to(dev)
        self.dB = torch.from_numpy(pk.bbuf.view(np.float64)).to(dev)
        self.dC = torch.zeros(pk.c_elems * (2 if pk.cplx else 1), dtype=torch.float64, device=dev)
        torch.cuda.synchronize(dev)
        self.pl = pk.pair_list()

    def run(self, prec="fp64", nslices=0, tol=1e-12, stats: dict | None = None):
        o = make_opts(prec, nslices, tol)
        st = Stats()
        check(self.ctx.lib.qs_grouped_gemm(self.ctx.h, C.byref(self.pl), C.c_void_p(self.dA.data_ptr()),
                                           C.c_void_p(self.dB.data_ptr()), C.c_void_p(self.dC.data_ptr()),
                                           C.byref(o), C.byref(st)))
        if stats is not None:
            stats.update(st.as_dict())

    def run_keyed(self, fkeys: np.ndarray, table: "FactorTable", prec="fp64", nslices=0, tol=1e-12,
                  stats: dict | None = None):
        """The batch with pair p's factor looked up on the device under the
        128-bit key fkeys[p] (uint64 array of shape (npairs, 2))."""
        k = np.ascontiguousarray(fkeys, dtype=np.uint64).reshape(-1, 2)
        if len(k) != self.pl.npairs:
            raise ValueError("one key per pair")
        o = make_opts(prec, nslices, tol)
        st = Stats()
        check(self.ctx.lib.qs_grouped_gemm_keyed(self.ctx.h, C.byref(self.pl), k.ctypes.data_as(C.c_void_p),
                                                 table.h, C.c_void_p(self.dA.data_ptr()),
                                                 C.c_void_p(self.dB.data_ptr()), C.c_void_p(self.dC.data_ptr()),
                                                 C.byref(o), C.byref(st)))
        if stats is not None:
            stats.update(st.as_dict())

    def plan(self, prec="split", nslices=0, tol=1e-12, autotune=False, graph=True) -> "GroupedPlan":
        return GroupedPlan(self.pk, prec, nslices, tol, autotune, graph, self.ctx)

    def run_plan(self, plan: "GroupedPlan", stats: dict | None = None):
        plan.run(self.dA.data_ptr(), self.dB.data_ptr(), self.dC.data_ptr(), stats)

    def result(self) -> list:
        self.ctx.sync()
        c = self.dC.cpu().numpy()
        if self.pk.cplx:
            c = c.view(np.complex128)
        return self.pk.unpack_c(c)


class GroupedPlan:
    """A reusable plan (qs_grouped_plan_*) over one pair list: planned once,
    replayed as a CUDA graph; ``autotune`` times the digit widths on the
    first run."""

    def __init__(self, pk: Packed, prec="split", nslices=0, tol=1e-12, autotune=False, graph=True,
                 ctx: Context | None = None):
        self.pk = pk
        self.ctx = ctx or default_context()
        flags = (_capi.QS_FLAG_AUTOTUNE if autotune else 0) | (0 if graph else _capi.QS_FLAG_NO_GRAPH)
        self.pl = pk.pair_list()
        h = C.c_void_p()
        check(self.ctx.lib.qs_grouped_plan_create(self.ctx.h, C.byref(self.pl),
                                                  C.byref(make_opts(prec, nslices, tol, flags)), C.byref(h)))
        self.h = h

    def run(self, dA: int, dB: int, dC: int, stats: dict | None = None):
        st = Stats()
        check(self.ctx.lib.qs_grouped_plan_run(self.h, C.c_void_p(dA), C.c_void_p(dB), C.c_void_p(dC),
                                               C.byref(st)))
        if stats is not None:
            stats.update(st.as_dict())

    def close(self):
        if getattr(self, "h", None):
            self.ctx.lib.qs_grouped_plan_destroy(self.h)
            self.h = None

    def __del__(self):
        self.close()


def run_device(w: dict, prec="fp64", nslices=0, tol=1e-12, ctx=None, stats=None) -> list:
    pk = Packed(w["A"], w["B"], w["afac"], cplx=w.get("complex"))
    db = DeviceBatch(pk, ctx)
    db.run(prec, nslices, tol, stats)
    return db.result()


class FactorTable:
    """Device-resident CG / X-symbol factors keyed by 128-bit keys
    (qs_xcache_*): the device form of the reference's X-symbol store (X3Map,
    Source/clebsch.hh:3911-4245).  Keys are uint64 arrays of shape (n, 2)."""

    def __init__(self, capacity: int, ctx: Context | None = None):
        self.ctx = ctx or default_context()
        h = C.c_void_p()
        check(self.ctx.lib.qs_xcache_create(self.ctx.h, int(capacity), C.byref(h)))
        self.h = h

    @staticmethod
    def _keys(keys) -> np.ndarray:
        return np.ascontiguousarray(keys, dtype=np.uint64).reshape(-1, 2)

    def put(self, keys, vals):
        k = self._keys(keys)
        v = np.ascontiguousarray(vals, dtype=np.float64).ravel()
        if len(v) != len(k):
            raise ValueError("one value per key")
        check(self.ctx.lib.qs_xcache_put(self.h, len(k), k.ctypes.data_as(C.c_void_p),
                                         v.ctypes.data_as(C.c_void_p)))

    def get(self, keys):
        """(values, found) looked up on the device."""
        k = self._keys(keys)
        v = np.zeros(len(k), np.float64)
        f = np.zeros(len(k), np.int32)
        check(self.ctx.lib.qs_xcache_get(self.h, len(k), k.ctypes.data_as(C.c_void_p),
                                         v.ctypes.data_as(C.c_void_p), f.ctypes.data_as(C.c_void_p)))
        return v, f.astype(bool)

    def __len__(self) -> int:
        n = C.c_int64()
        check(self.ctx.lib.qs_xcache_count(self.h, C.byref(n)))
        return int(n.value)

    def close(self):
        if self.h:
            self.ctx.lib.qs_xcache_destroy(self.h)
            self.h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass
