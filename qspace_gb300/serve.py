"""Serving loop: continuous batching of contractQS requests between
device-resident tensors (qs_server_* of the C-ABI).

Many NRG z-shift / DMRG instances submit contractions as requests; the
server admits them onto slot streams as slots and HBM budget free up, so
requests arriving while others run overlap on the device.  Each result is
identical to the same contraction run alone (deterministic kernels, no
shared buffers).
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

    def submit(self, A: Tensor, ia, B: Tensor, ib, perm=None, prec: str = "fp64", nslices: int = 0,
               tol: float = 1e-12) -> int:
        p, n = _perm_arg(perm)
        o = make_opts(prec, nslices, tol)
        t = C.c_int64()
        check(self.ctx.lib.qs_server_submit(self.h, A.h, _idx_str(ia), B.h, _idx_str(ib), p, n, C.byref(o),
                                            C.byref(t)))
        return t.value

    def poll(self, ticket: int, timeout_ms: int = 0):
        """(done, Tensor or None, latency_ms).  Raises QSError for a failed or
        cancelled request."""
        done, lat = C.c_int32(), C.c_double()
        h = C.c_void_p()
        check(self.ctx.lib.qs_server_poll(self.h, int(ticket), int(timeout_ms), C.byref(done), C.byref(h),
                                          C.byref(lat)))
        if not done.value:
            return False, None, None
        return True, Tensor(self.ctx, h), lat.value

    def wait(self, ticket: int, timeout_s: float = 60.0):
        import time
        t0 = time.monotonic()
        while True:
            done, T, lat = self.poll(ticket, 50)
            if done:
                return T, lat
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
