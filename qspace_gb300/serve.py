"""Serving loop: continuous batching of contractQS and eigQS requests on
device-resident tensors (qs_server_* of the C-ABI).

Many NRG z-shift / DMRG instances submit their contractions and block
eigendecompositions as requests; the server admits them onto slot streams
as slots and HBM budget free up, so requests arriving while others run
overlap on the device.  Each result is identical to the same operation run
alone (deterministic kernels, no shared buffers).
"""
from __future__ import annotations

import ctypes as C

from . import _capi
from ._capi import QSError, ServerCfg, check
from .qspace import Context, Tensor, _idx_str, _perm_arg, default_context, make_opts


class Server:
    def __init__(self, nslots: int = 4, hbm_budget: int = 8 << 30, ctx: Context | None = None,
                 max_batch: int = 0):
        self.ctx = ctx or default_context()
        cfg = ServerCfg()
        cfg.nslots = nslots
        cfg.max_batch = max_batch
        cfg.hbm_budget = int(hbm_budget)
        h = C.c_void_p()
        check(self.ctx.lib.qs_server_create(self.ctx.h, C.byref(cfg), C.byref(h)))
        self.h = h
        self._eig_sizes = {}   # ticket -> H of pending eig requests
        self._owner = {}       # ticket -> context that owns the result

    def submit(self, A: Tensor, ia, B: Tensor, ib, perm=None, prec: str = "fp64", nslices: int = 0,
               tol: float = 1e-12, client: Context | None = None) -> int:
        """Enqueue contractQS(A, ia, B, ib [,perm]).  With `client` (the
        submitter's own context) the request is ordered after the client's
        stream and its result belongs to the client's context
        (qs_server_submit_from); otherwise to the server's."""
        p, n = _perm_arg(perm)
        o = make_opts(prec, nslices, tol)
        t = C.c_int64()
        check(self.ctx.lib.qs_server_submit_from(self.h, client.h if client else None, A.h, _idx_str(ia), B.h,
                                                 _idx_str(ib), p, n, C.byref(o), C.byref(t)))
        self._owner[t.value] = client or self.ctx
        return t.value

    def poll(self, ticket: int, timeout_ms: int = 0):
        """(done, Tensor or None, latency_ms).  Raises QSError for a failed or
        cancelled request."""
        done, lat = C.c_int32(), C.c_double()
        h = C.c_void_p()
        try:
            check(self.ctx.lib.qs_server_poll(self.h, int(ticket), int(timeout_ms), C.byref(done), C.byref(h),
                                              C.byref(lat)))
        except QSError:
            self._owner.pop(ticket, None)
            raise
        if not done.value:
            return False, None, None
        return True, Tensor(self._owner.pop(ticket, self.ctx), h), lat.value

    def wait(self, ticket: int, timeout_s: float = 60.0):
        import time
        t0 = time.monotonic()
        while True:
            done, T, lat = self.poll(ticket, 50)
            if done:
                return T, lat
            if time.monotonic() - t0 > timeout_s:
                raise QSError(6, f"request {ticket} did not complete in {timeout_s} s")

    def submit_eig(self, H: Tensor, nkeep: int = -1, etrunc: float = 0.0, deps: float = 0.0,
                   client: Context | None = None) -> int:
        """Enqueue eigQS(H, 'Nkeep', nkeep, 'Etrunc', etrunc) of a device
        tensor (qs_server_submit_eig_from; `client` as for submit).  H must
        stay alive until the result is collected."""
        t = C.c_int64()
        check(self.ctx.lib.qs_server_submit_eig_from(self.h, client.h if client else None, H.h, int(nkeep),
                                                     float(etrunc), float(deps), C.byref(t)))
        self._eig_sizes[t.value] = H
        self._owner[t.value] = client or self.ctx
        return t.value

    def poll_eig(self, ticket: int, timeout_ms: int = 0):
        """(done, result dict or None).  The dict holds AK / AD (device
        tensors of the kept / discarded eigenvectors), E and keep (host arrays
        in H's block order), NK, Etrunc and the latency in ms."""
        import numpy as np
        H = self._eig_sizes[ticket]
        rank, qdim, nblk, _, _ = H.meta()
        dims = np.empty(max(nblk * rank, 1), np.int64)
        check(self.ctx.lib.qs_tensor_meta(H.h, None, dims.ctypes.data_as(_capi.c_int64_p), None))
        ntot = int(dims[:nblk * rank:rank].sum()) if nblk else 0
        E = np.zeros(max(ntot, 1))
        keep = np.zeros(max(ntot, 1), np.uint8)
        done, lat, et = C.c_int32(), C.c_double(), C.c_double()
        nk = C.c_int64()
        ak, ad = C.c_void_p(), C.c_void_p()
        try:
            check(self.ctx.lib.qs_server_poll_eig(self.h, int(ticket), int(timeout_ms), C.byref(done), C.byref(ak),
                                                  C.byref(ad), E.ctypes.data_as(_capi.c_double_p),
                                                  keep.ctypes.data_as(C.POINTER(C.c_uint8)), C.byref(nk),
                                                  C.byref(et), C.byref(lat)))
        except QSError:
            self._eig_sizes.pop(ticket, None)
            self._owner.pop(ticket, None)
            raise
        if not done.value:
            return False, None
        self._eig_sizes.pop(ticket, None)
        owner = self._owner.pop(ticket, self.ctx)
        return True, {"AK": Tensor(owner, ak), "AD": Tensor(owner, ad), "E": E[:ntot],
                      "keep": keep[:ntot].astype(bool), "NK": nk.value, "Etrunc": et.value,
                      "latency_ms": lat.value}

    def wait_eig(self, ticket: int, timeout_s: float = 120.0) -> dict:
        import time
        t0 = time.monotonic()
        while True:
            done, r = self.poll_eig(ticket, 50)
            if done:
                return r
            if time.monotonic() - t0 > timeout_s:
                raise QSError(6, f"request {ticket} did not complete in {timeout_s} s")

    def cancel(self, ticket: int):
        check(self.ctx.lib.qs_server_cancel(self.h, int(ticket)))

    def close(self):
        if getattr(self, "h", None):
            self.ctx.lib.qs_server_destroy(self.h)
            self.h = None

    def __enter__(self):
        return self

    def __exit__(self, *exc):
        self.close()

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass
