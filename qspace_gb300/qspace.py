"""Host-side mirror of QSpace's MEX interface on top of libqsgpu.

``QSpace`` mirrors the MATLAB struct ``{Q, data, info}`` (Source/QSpace.hh:
3092): ``Q`` is a list with one (nblk x qdim) int array per leg, ``data`` a
list of dense blocks, ``info`` a dict (``itags``).  The functions keep the
reference's names, argument meaning and error behaviour:

* ``contractQS(A, ia, B, ib[, perm])`` -- Source/contractQS.cc:505-632;
* ``permuteQS(A, perm[, 'conj'])``     -- Source/permuteQS.cc:198-258.

All numerical work, label matching and itag bookkeeping run in the library
behind the C-ABI; this module only packs and unpacks host buffers.
``Tensor`` is a device-resident QSpace.
"""
from __future__ import annotations

import ctypes as C
import threading
from dataclasses import dataclass, field

import numpy as np

from . import _capi
from ._capi import QSError, QSpaceView, Opts, Stats, check

__all__ = ["QSpace", "Tensor", "Context", "contractQS", "permuteQS", "default_context",
           "upload", "contract_dev", "permute_dev", "to_wire", "from_wire", "upload_wire", "plus_dev", "plusQS"]


# --------------------------------------------------------------------- QSpace
@dataclass
class QSpace:
    Q: list                      # per leg: (nblk, qdim) int32
    data: list                   # per block: ndarray with the leg dims
    info: dict = field(default_factory=dict)

    @property
    def rank(self) -> int:
        return len(self.Q)

    @property
    def nblk(self) -> int:
        return len(self.data)

    @property
    def qdim(self) -> int:
        if not self.Q or self.nblk == 0:
            return 1
        return int(np.asarray(self.Q[0]).reshape(self.nblk, -1).shape[1])

    @property
    def is_complex(self) -> bool:
        return any(np.iscomplexobj(d) for d in self.data)

    def block_dims(self, i: int) -> tuple:
        r = self.rank
        s = tuple(int(x) for x in np.shape(self.data[i]))
        if len(s) > r:
            if any(x != 1 for x in s[r:]):
                raise ValueError("block has more non-singleton dims than legs")
            s = s[:r]
        return s + (1,) * (r - len(s))

    @classmethod
    def from_dict(cls, d: dict) -> "QSpace":
        return cls([np.asarray(q, dtype=np.int32).reshape(len(q), -1) if np.ndim(q) else q
                    for q in d["Q"]], list(d["data"]), dict(d.get("info") or {}))

    def to_dict(self) -> dict:
        return {"Q": [np.asarray(q) for q in self.Q], "data": list(self.data), "info": dict(self.info)}

    # -- packing into the C-ABI layout
    def pack(self):
        """(view, keepalive): labels block-major int32, dims int64, blocks
        column-major back to back (complex interleaved)."""
        n, r = self.nblk, self.rank
        qd = self.qdim
        cplx = self.is_complex
        if n and r:
            q = np.stack([np.asarray(x, dtype=np.int32).reshape(n, qd) for x in self.Q], axis=1)
            q = np.ascontiguousarray(q.reshape(n, r * qd), dtype=np.int32)
        else:
            q = np.zeros((0,), np.int32)
        dims = np.array([self.block_dims(i) for i in range(n)], dtype=np.int64).reshape(n, r)
        sizes = np.prod(dims, axis=1) if r else np.ones(n, np.int64)
        offs = np.zeros(n, np.int64)
        if n > 1:
            offs[1:] = np.cumsum(sizes)[:-1]
        total = int(sizes.sum()) if n else 0
        buf = np.empty(total, dtype=np.complex128 if cplx else np.float64)
        for i, d in enumerate(self.data):
            a = np.asarray(d, dtype=buf.dtype)
            buf[offs[i]:offs[i] + sizes[i]] = a.reshape(-1, order="F") if a.ndim > 1 else a.reshape(-1)
        dims = np.ascontiguousarray(dims)
        v = QSpaceView()
        v.rank, v.qdim, v.nblk = r, qd, n
        v.q = q.ctypes.data_as(_capi.c_int32_p)
        v.dims = dims.ctypes.data_as(_capi.c_int64_p)
        v.offs = offs.ctypes.data_as(_capi.c_int64_p)
        v.data = buf.ctypes.data_as(_capi.c_double_p)
        v.is_complex = 1 if cplx else 0
        tags = self.info.get("itags")
        tb = ",".join(tags).encode() if tags else None
        v.itags = tb
        return v, (q, dims, offs, buf, tb)

    @classmethod
    def unpack(cls, rank, qdim, q, dims, offs, data, cplx, info=None) -> "QSpace":
        n = len(offs)
        if n == 0:
            return cls([], [], dict(info or {}))
        q = np.asarray(q, np.int32).reshape(n, rank, qdim)
        dims = np.asarray(dims, np.int64).reshape(n, rank)
        arr = np.asarray(data)
        if cplx:
            arr = arr.view(np.complex128)
        blocks = []
        for i in range(n):
            s = int(np.prod(dims[i])) if rank else 1
            blk = arr[offs[i]:offs[i] + s]
            blocks.append(blk.reshape(tuple(dims[i]), order="F") if rank else blk.reshape(()))
        Q = [np.ascontiguousarray(q[:, k, :]) for k in range(rank)]
        return cls(Q, blocks, dict(info or {}))


# -------------------------------------------------------------------- context
class Context:
    """One CUDA device + stream + memory pool (qs_ctx)."""

    def __init__(self, device: int = 0):
        self.lib = _capi.load()
        h = C.c_void_p()
        check(self.lib.qs_ctx_create(device, C.byref(h)))
        self.h = h
        self.device = device

    @property
    def stream_ptr(self) -> int:
        return int(self.lib.qs_ctx_stream(self.h) or 0)

    @property
    def launches(self) -> int:
        return int(self.lib.qs_ctx_launches(self.h))

    def sync(self):
        check(self.lib.qs_ctx_sync(self.h))

    def set_timing(self, on: bool = True):
        check(self.lib.qs_ctx_set_timing(self.h, 1 if on else 0))

    def phase_ms(self) -> tuple[float, float]:
        """(operand preparation ms, GEMM kernel ms) of the most recent call."""
        a, b = C.c_double(), C.c_double()
        check(self.lib.qs_ctx_phase_ms(self.h, C.byref(a), C.byref(b)))
        return a.value, b.value

    def close(self):
        if getattr(self, "h", None):
            self.lib.qs_ctx_destroy(self.h)
            self.h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass


_ctx_lock = threading.Lock()
_contexts: dict[int, Context] = {}


def default_context(device: int = 0) -> Context:
    with _ctx_lock:
        c = _contexts.get(device)
        if c is None:
            c = _contexts[device] = Context(device)
        return c


def make_opts(prec: str = "fp64", nslices: int = 0, tol: float = 1e-12, flags: int = 0) -> Opts:
    o = Opts()
    p = prec.lower()
    if p in ("fp64", "plain", "double"):
        o.prec = _capi.QS_PREC_FP64
    elif p in ("split", "bf16", "ozaki"):
        o.prec = _capi.QS_PREC_SPLIT
    else:
        raise ValueError(f"unknown precision mode '{prec}'")
    o.nslices, o.tol, o.flags = int(nslices), float(tol), int(flags)
    return o


def _perm_list(perm) -> list:
    """1-based permutation as a list of ints ('312', '3,1,2' or a sequence)."""
    if isinstance(perm, str):
        s = perm.strip()
        if any(c in s for c in ",; "):
            return [int(x) for x in s.replace(",", " ").replace(";", " ").split()]
        return [int(c) for c in s]
    return [int(x) for x in np.atleast_1d(perm)]


def _perm_arg(perm):
    if perm is None:
        return None, 0
    if isinstance(perm, str):
        s = perm.strip()
        if not s:
            return None, 0
        if any(c in s for c in ",; "):
            p = [int(x) for x in s.replace(",", " ").replace(";", " ").split()]
        else:
            p = [int(c) for c in s]
    else:
        p = [int(x) for x in np.atleast_1d(perm)]
    if not p:
        return None, 0
    arr = (C.c_int32 * len(p))(*p)
    return arr, len(p)


def _idx_str(ix) -> bytes:
    if isinstance(ix, str):
        return ix.encode()
    v = [int(x) for x in np.atleast_1d(ix)]
    # numeric (1-based) indices: bracketed and blank separated so that a
    # single multi-digit leg is not read in compact form
    return ("[" + " ".join(str(x) for x in v) + " ]").encode()


# ---------------------------------------------------------------- host calls
def _result_to_qspace(lib, res, info=None) -> QSpace:
    r, qd, nb, ne, cx = C.c_int32(), C.c_int32(), C.c_int64(), C.c_int64(), C.c_int32()
    check(lib.qs_result_info(res, C.byref(r), C.byref(qd), C.byref(nb), C.byref(ne), C.byref(cx)))
    n, rank, qdim = nb.value, r.value, qd.value
    q = np.empty(max(n * rank * qdim, 1), np.int32)
    dims = np.empty(max(n * rank, 1), np.int64)
    offs = np.empty(max(n, 1), np.int64)
    data = np.empty(max(ne.value * (2 if cx.value else 1), 1), np.float64)
    check(lib.qs_result_copy(res, q.ctypes.data_as(_capi.c_int32_p), dims.ctypes.data_as(_capi.c_int64_p),
                             offs.ctypes.data_as(_capi.c_int64_p), data.ctypes.data_as(_capi.c_double_p)))
    tb = C.create_string_buffer(4096)
    check(lib.qs_result_itags(res, tb, 4096))
    lib.qs_result_free(res)
    if tb.value:
        info = dict(info or {})
        info["itags"] = tb.value.decode().split(",")
    return QSpace.unpack(rank, qdim, q[:n * rank * qdim], dims[:n * rank], offs[:n], data, bool(cx.value), info)


def contractQS(A, ia=None, B: QSpace | None = None, ib=None, perm=None, *, prec: str = "fp64", nslices: int = 0,
               tol: float = 1e-12, ctx: Context | None = None, stats: dict | None = None) -> QSpace:
    """C = contractQS(A, ia, B, ib [,perm]) on the GPU (host buffers in/out).

    ``ia``/``ib``: '12*' style strings or 1-based sequences; ``perm`` 1-based.
    ``prec``: 'fp64' (plain drop-in) or 'split' (BF16 digits on tcgen05).

    Cell form ``contractQS([X0, X1, '*', X2, ...] [, perm])``: contraction
    over matching itags, right to left (Source/contractQS.cc:634-808); a '*'
    after a QSpace is its conj option.
    """
    if isinstance(A, (list, tuple)):
        return contract_itags(A, ia, prec=prec, nslices=nslices, tol=tol, ctx=ctx)
    ctx = ctx or default_context()
    va, ka = A.pack()
    vb, kb = B.pack()
    p, n = _perm_arg(perm)
    o = make_opts(prec, nslices, tol)
    st = Stats()
    res = C.c_void_p()
    check(ctx.lib.qs_contractQS(ctx.h, C.byref(va), _idx_str(ia), C.byref(vb), _idx_str(ib), p, n,
                                C.byref(o), C.byref(res), C.byref(st)))
    out = _result_to_qspace(ctx.lib, res, None)
    if stats is not None:
        stats.update(st.as_dict())
    del ka, kb
    return out


def permuteQS(A: QSpace, perm, conj=False, *, ctx: Context | None = None) -> QSpace:
    """permuteQS(A, perm [,'conj']) on the GPU; block order unchanged."""
    ctx = ctx or default_context()
    if isinstance(conj, str):
        conj = conj.lower() == "conj"
    va, ka = A.pack()
    p, n = _perm_arg(perm)
    res = C.c_void_p()
    check(ctx.lib.qs_permuteQS(ctx.h, C.byref(va), p, n, 1 if conj else 0, C.byref(res)))
    info = {k: v for k, v in A.info.items() if k != "itags"}
    return _result_to_qspace(ctx.lib, res, info)


# ------------------------------------------------------------ device tensors
class Tensor:
    """A device-resident QSpace (qs_tensor)."""

    def __init__(self, ctx: Context, handle: C.c_void_p, info: dict | None = None):
        self.ctx, self.h, self.info = ctx, handle, dict(info or {})

    def meta(self):
        r, qd, nb, ne, cx = C.c_int32(), C.c_int32(), C.c_int64(), C.c_int64(), C.c_int32()
        check(self.ctx.lib.qs_tensor_info(self.h, C.byref(r), C.byref(qd), C.byref(nb), C.byref(ne),
                                          C.byref(cx)))
        return r.value, qd.value, nb.value, ne.value, bool(cx.value)

    @property
    def data_ptr(self) -> int:
        return int(self.ctx.lib.qs_tensor_data(self.h) or 0)

    def download(self) -> QSpace:
        rank, qdim, n, ne, cx = self.meta()
        q = np.empty(max(n * rank * qdim, 1), np.int32)
        dims = np.empty(max(n * rank, 1), np.int64)
        offs = np.empty(max(n, 1), np.int64)
        data = np.empty(max(ne * (2 if cx else 1), 1), np.float64)
        check(self.ctx.lib.qs_tensor_download(self.ctx.h, self.h, q.ctypes.data_as(_capi.c_int32_p),
                                              dims.ctypes.data_as(_capi.c_int64_p),
                                              offs.ctypes.data_as(_capi.c_int64_p),
                                              data.ctypes.data_as(_capi.c_double_p)))
        tb = C.create_string_buffer(4096)
        check(self.ctx.lib.qs_tensor_itags(self.h, tb, 4096))
        info = dict(self.info)
        if tb.value:
            info["itags"] = tb.value.decode().split(",")
        return QSpace.unpack(rank, qdim, q[:n * rank * qdim], dims[:n * rank], offs[:n], data, cx, info)

    def to_wire(self) -> np.ndarray:
        """The tensor as a wire container (qs_tensor_to_wire: its device data
        copied once, straight into the container's data section)."""
        n = C.c_int64()
        check(self.ctx.lib.qs_tensor_wire_size(self.h, C.byref(n)))
        buf = np.empty(n.value, np.uint8)
        check(self.ctx.lib.qs_tensor_to_wire(self.ctx.h, self.h, buf.ctypes.data_as(C.c_void_p), n.value))
        return buf

    def free(self):
        if self.h:
            self.ctx.lib.qs_tensor_free(self.h)
            self.h = None

    def __del__(self):
        try:
            self.free()
        except Exception:
            pass


# ------------------------------------------------------------ wire container
def to_wire(A: QSpace) -> np.ndarray:
    """Pack a QSpace into one flat binary container (qs_wire_pack); returns a
    uint8 array (64-byte aligned) that can be written, sent or memory-mapped."""
    lib = _capi.load()
    v, keep = A.pack()
    n = C.c_int64()
    check(lib.qs_wire_size(C.byref(v), C.byref(n)))
    buf = np.empty(n.value, np.uint8)
    check(lib.qs_wire_pack(C.byref(v), buf.ctypes.data_as(C.c_void_p), n.value))
    del keep
    return buf


def _aligned(buf) -> np.ndarray:
    a = np.frombuffer(buf, np.uint8)
    if a.ctypes.data % 8:
        a = a.copy()   # the container's sections are read in place: 8-byte alignment
    return a


def from_wire(buf) -> QSpace:
    """Read a container without copying its data: the blocks of the returned
    QSpace are read-only numpy views into ``buf`` (qs_wire_view validates
    the container first)."""
    lib = _capi.load()
    a = _aligned(buf)
    v = QSpaceView()
    check(lib.qs_wire_view(a.ctypes.data_as(C.c_void_p), a.size, C.byref(v)))
    base = a.ctypes.data
    n, r, qd = v.nblk, v.rank, v.qdim

    def at(ptr, dtype, count):
        off = C.cast(ptr, C.c_void_p).value - base if count else 0
        return np.frombuffer(a, dtype, count, off) if count else np.zeros(0, dtype)

    q = at(v.q, np.int32, n * r * qd)
    dims = at(v.dims, np.int64, n * r)
    offs = at(v.offs, np.int64, n)
    ext = int(max((offs[i] + int(np.prod(dims[i * r:(i + 1) * r])) for i in range(n)), default=0)) if n else 0
    data = at(v.data, np.float64, ext * (2 if v.is_complex else 1))
    info = {"itags": v.itags.decode().split(",")} if v.itags else {}
    if n == 0:
        return QSpace([np.zeros((0, qd), np.int32) for _ in range(r)], [], info)
    return QSpace.unpack(r, qd, q, dims, offs, data, bool(v.is_complex), info)


def upload_wire(buf, ctx: Context | None = None, info: dict | None = None) -> Tensor:
    """Device tensor straight from a container (one host->device copy of
    its data section; qs_tensor_from_wire)."""
    ctx = ctx or default_context()
    a = _aligned(buf)
    h = C.c_void_p()
    check(ctx.lib.qs_tensor_from_wire(ctx.h, a.ctypes.data_as(C.c_void_p), a.size, C.byref(h)))
    ctx.sync()
    return Tensor(ctx, h, info)


def upload(A: QSpace, ctx: Context | None = None) -> Tensor:
    ctx = ctx or default_context()
    v, keep = A.pack()
    h = C.c_void_p()
    check(ctx.lib.qs_tensor_upload(ctx.h, C.byref(v), C.byref(h)))
    ctx.sync()
    del keep
    return Tensor(ctx, h, A.info)


def upload_packed(q, dims, buf, ctx: Context | None = None, info: dict | None = None) -> Tensor:
    """Device tensor from the packed form directly (no per-block Python
    objects): q (nblk, rank, qdim) int32 labels, dims (nblk, rank) int64,
    buf the blocks column-major back to back (float64 or complex128)."""
    ctx = ctx or default_context()
    q = np.ascontiguousarray(q, np.int32)
    n, r = int(q.shape[0]), int(q.shape[1])
    qd = int(q.shape[2]) if q.ndim == 3 else 1
    dims = np.ascontiguousarray(dims, np.int64).reshape(n, r)
    sizes = np.prod(dims, axis=1) if r else np.ones(n, np.int64)
    offs = np.zeros(n, np.int64)
    if n > 1:
        offs[1:] = np.cumsum(sizes)[:-1]
    buf = np.ascontiguousarray(buf)
    if buf.size != int(sizes.sum()):
        raise ValueError("upload_packed: buffer size does not match the block dimensions")
    cplx = np.iscomplexobj(buf)
    v = _capi.QSpaceView()
    v.rank, v.qdim, v.nblk = r, qd, n
    v.q = q.ctypes.data_as(_capi.c_int32_p)
    v.dims = dims.ctypes.data_as(_capi.c_int64_p)
    v.offs = offs.ctypes.data_as(_capi.c_int64_p)
    v.data = buf.view(np.float64).ctypes.data_as(_capi.c_double_p)
    v.is_complex = 1 if cplx else 0
    tags = (info or {}).get("itags")
    tb = ",".join(tags).encode() if tags else None
    v.itags = tb
    h = C.c_void_p()
    check(ctx.lib.qs_tensor_upload(ctx.h, C.byref(v), C.byref(h)))
    ctx.sync()
    return Tensor(ctx, h, info)


def contract_dev(A: Tensor, ia, B: Tensor, ib, perm=None, *, prec: str = "fp64", nslices: int = 0,
                 tol: float = 1e-12, stats: dict | None = None) -> Tensor:
    ctx = A.ctx
    p, n = _perm_arg(perm)
    o = make_opts(prec, nslices, tol)
    st = Stats()
    h = C.c_void_p()
    check(ctx.lib.qs_contract_dev(ctx.h, A.h, _idx_str(ia), B.h, _idx_str(ib), p, n, C.byref(o),
                                  C.byref(h), C.byref(st)))
    if stats is not None:
        stats.update(st.as_dict())
    return Tensor(ctx, h)


def plus_dev(A: Tensor, B: Tensor, bfac: float = 1.0) -> Tensor:
    """plusQS of device tensors: A + bfac * B (qs_plus_dev)."""
    ctx = A.ctx
    h = C.c_void_p()
    check(ctx.lib.qs_plus_dev(ctx.h, A.h, B.h, float(bfac), C.byref(h)))
    return Tensor(ctx, h)


def plusQS(A: QSpace, B: QSpace, bfac: float = 1.0, ctx: Context | None = None) -> QSpace:
    """plusQS(A, B [,bfac]) with host QSpaces (through the device)."""
    ctx = ctx or default_context()
    ta, tb = upload(A, ctx), upload(B, ctx)
    try:
        tc = plus_dev(ta, tb, bfac)
        try:
            return tc.download()
        finally:
            tc.free()
    finally:
        ta.free()
        tb.free()


def contract_batch(jobs, *, prec: str = "fp64", nslices: int = 0, tol: float = 1e-12) -> list:
    """Device-resident contractions [(A, ia, B, ib[, perm]), ...] whose block
    products share one grouped launch (qs_contract_batch).  Returns Tensors."""
    if not jobs:
        return []
    ctx = jobs[0][0].ctx
    n = len(jobs)
    A = (C.c_void_p * n)(*[j[0].h.value for j in jobs])
    B = (C.c_void_p * n)(*[j[2].h.value for j in jobs])
    ia = (C.c_char_p * n)(*[_idx_str(j[1]) for j in jobs])
    ib = (C.c_char_p * n)(*[_idx_str(j[3]) for j in jobs])
    perms = [np.asarray(_perm_list(j[4]) if len(j) > 4 and j[4] is not None else [], np.int32) for j in jobs]
    P = (_capi.c_int32_p * n)(*[p.ctypes.data_as(_capi.c_int32_p) if p.size else None for p in perms])
    NP = np.array([p.size for p in perms], np.int32)
    out = (C.c_void_p * n)()
    check(ctx.lib.qs_contract_batch(ctx.h, n, A, ia, B, ib, P, NP.ctypes.data_as(_capi.c_int32_p),
                                    C.byref(make_opts(prec, nslices, tol)), out))
    return [Tensor(ctx, C.c_void_p(out[r])) for r in range(n)]


def _cell_items(items):
    """[X0, '*', X1, ...] -> [(X0, conj0), (X1, conj1), ...]"""
    out = []
    for x in items:
        if isinstance(x, str):
            if not out or x.strip() != "*":
                raise QSError(1, f"invalid cell-contraction option {x!r}")
            out[-1] = (out[-1][0], not out[-1][1])
        else:
            out.append((x, False))
    return out


def contract_itags(items, perm=None, *, prec: str = "fp64", nslices: int = 0, tol: float = 1e-12,
                   ctx: Context | None = None):
    """Cell contraction over matching itags (qs_contract_itags).  Items are
    QSpace (host; result returned as QSpace) or Tensor (device; result
    returned as Tensor), each optionally followed by '*'."""
    pairs = _cell_items(items)
    dev = all(isinstance(x, Tensor) for x, _ in pairs)
    if not dev and any(isinstance(x, Tensor) for x, _ in pairs):
        raise QSError(1, "cell contraction mixes host and device tensors")
    ctx = pairs[0][0].ctx if dev else (ctx or default_context())
    T = [x if dev else upload(x, ctx) for x, _ in pairs]
    arr = (C.c_void_p * len(T))(*[t.h.value for t in T])
    conj = np.array([1 if c else 0 for _, c in pairs], np.int32)
    p, n = _perm_arg(perm)
    o = make_opts(prec, nslices, tol)
    h = C.c_void_p()
    check(ctx.lib.qs_contract_itags(ctx.h, len(T), arr, conj.ctypes.data_as(_capi.c_int32_p), p, n,
                                    C.byref(o), C.byref(h)))
    R = Tensor(ctx, h)
    return R if dev else R.download()


def permute_dev(A: Tensor, perm, conj=False) -> Tensor:
    ctx = A.ctx
    p, n = _perm_arg(perm)
    h = C.c_void_p()
    check(ctx.lib.qs_permute_dev(ctx.h, A.h, p, n, 1 if conj else 0, C.byref(h)))
    return Tensor(ctx, h)
