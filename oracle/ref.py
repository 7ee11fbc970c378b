"""ctypes driver of the reference oracle (test infrastructure only).

Calls the reference's own MEX entry points (contractQS, permuteQS, ...),
compiled unmodified into oracle/_ref/<name>.so against the fake MATLAB
runtime (oracle/refshim, oracle/refbuild.py).  Inputs and outputs are the
QSpace dicts of oracle/qs_oracle.py ({'Q': [...], 'data': [...], 'info':
{...}}); QSpaces travel as MATLAB structs {Q, data, info}
(Source/QSpace.hh:3092), with labels as double matrices and blocks as
column-major double / complex arrays, exactly as MATLAB would pass them.

Only available where the reference sources were present at build time (this
is never the GPU machine): ``available()`` tells.
"""
from __future__ import annotations

import ctypes as C
import os
from pathlib import Path

import numpy as np

HERE = Path(__file__).resolve().parent
REF = HERE / "_ref"

mxREAL, mxCOMPLEX = 0, 1
mxDOUBLE_CLASS = 6
_lib = None
_mex = {}


def available(name: str = "contractQS") -> bool:
    return (REF / "libfakemx.so").exists() and (REF / f"{name}.so").exists()


def _fake():
    global _lib
    if _lib is None:
        lib = C.CDLL(str(REF / "libfakemx.so"), mode=os.RTLD_NOW | C.RTLD_GLOBAL)
        vp, sz, i32 = C.c_void_p, C.c_size_t, C.c_int
        sig = {
            "mxCreateStructMatrix": (vp, [sz, sz, i32, C.POINTER(C.c_char_p)]),
            "mxCreateCellMatrix": (vp, [sz, sz]),
            "mxCreateDoubleMatrix": (vp, [sz, sz, i32]),
            "mxCreateNumericArray": (vp, [sz, C.POINTER(sz), i32, i32]),
            "mxCreateString": (vp, [C.c_char_p]),
            "mxSetCell": (None, [vp, sz, vp]),
            "mxGetCell": (vp, [vp, sz]),
            "mxSetFieldByNumber": (None, [vp, sz, i32, vp]),
            "mxGetField": (vp, [vp, sz, C.c_char_p]),
            "mxGetData": (vp, [vp]),
            "mxGetM": (sz, [vp]),
            "mxGetN": (sz, [vp]),
            "mxGetNumberOfElements": (sz, [vp]),
            "mxGetNumberOfDimensions": (sz, [vp]),
            "mxGetDimensions": (C.POINTER(sz), [vp]),
            "mxIsComplex": (C.c_bool, [vp]),
            "mxIsCell": (C.c_bool, [vp]),
            "mxIsChar": (C.c_bool, [vp]),
            "mxIsStruct": (C.c_bool, [vp]),
            "mxGetString": (i32, [vp, C.c_char_p, sz]),
            "mxDestroyArray": (None, [vp]),
            "fakemx_call": (i32, [vp, C.c_char_p, i32, C.POINTER(vp), i32, C.POINTER(vp)]),
            "fakemx_last_error": (C.c_char_p, []),
        }
        for k, (r, a) in sig.items():
            f = getattr(lib, k)
            f.restype, f.argtypes = r, a
        _lib = lib
    return _lib


def _mexfn(name: str):
    if name not in _mex:
        so = C.CDLL(str(REF / f"{name}.so"), mode=os.RTLD_NOW | C.RTLD_LOCAL)
        _mex[name] = (so, C.cast(so.mexFunction, C.c_void_p))
    return _mex[name][1]


class RefError(RuntimeError):
    pass


# ------------------------------------------------------------ conversion
def _mx_array(x: np.ndarray):
    lib = _fake()
    x = np.asarray(x)
    cplx = np.iscomplexobj(x)
    dims = x.shape if x.ndim >= 2 else (x.shape + (1,) * (2 - x.ndim))
    d = (C.c_size_t * len(dims))(*dims)
    a = lib.mxCreateNumericArray(len(dims), d, mxDOUBLE_CLASS, mxCOMPLEX if cplx else mxREAL)
    flat = np.asfortranarray(x.astype(np.complex128 if cplx else np.float64)).reshape(-1, order="F")
    if flat.size:
        C.memmove(lib.mxGetData(a), flat.ctypes.data, flat.nbytes)
    return a


def _mx_string(s: str):
    return _fake().mxCreateString(s.encode())


def to_mx(A: dict):
    """QSpace dict -> MATLAB struct {Q, data, info}."""
    lib = _fake()
    names = (C.c_char_p * 3)(b"Q", b"data", b"info")
    S = lib.mxCreateStructMatrix(1, 1, 3, names)
    r = len(A["Q"])
    n = len(A["data"])
    Qc = lib.mxCreateCellMatrix(1, r)
    for k in range(r):
        q = np.asarray(A["Q"][k], dtype=np.float64)
        q = q.reshape(n, -1) if n else q.reshape(0, q.shape[-1] if q.ndim == 2 else 1)
        lib.mxSetCell(Qc, k, _mx_array(q))
    D = lib.mxCreateCellMatrix(n, 1)
    for i, blk in enumerate(A["data"]):
        lib.mxSetCell(D, i, _mx_array(np.asarray(blk)))
    info = (A.get("info") or {})
    if info.get("itags"):
        fn = (C.c_char_p * 1)(b"itags")
        I = lib.mxCreateStructMatrix(1, 1, 1, fn)
        tags = lib.mxCreateCellMatrix(1, len(info["itags"]))
        for k, t in enumerate(info["itags"]):
            lib.mxSetCell(tags, k, _mx_string(t))
        lib.mxSetFieldByNumber(I, 0, 0, tags)
    else:
        I = lib.mxCreateDoubleMatrix(0, 0, mxREAL)
    lib.mxSetFieldByNumber(S, 0, 0, Qc)
    lib.mxSetFieldByNumber(S, 0, 1, D)
    lib.mxSetFieldByNumber(S, 0, 2, I)
    return S


def _np_of(a) -> np.ndarray:
    lib = _fake()
    nd = lib.mxGetNumberOfDimensions(a)
    dp = lib.mxGetDimensions(a)
    dims = tuple(int(dp[i]) for i in range(nd))
    n = int(np.prod(dims))
    cplx = bool(lib.mxIsComplex(a))
    buf = (C.c_double * (n * (2 if cplx else 1))).from_address(lib.mxGetData(a)) if n else []
    arr = np.array(buf, dtype=np.float64)
    if cplx:
        arr = arr.view(np.complex128)
    return arr.reshape(dims, order="F")


def _str_of(a) -> str:
    lib = _fake()
    buf = C.create_string_buffer(256)
    lib.mxGetString(a, buf, 256)
    return buf.value.decode()


def from_mx(S) -> dict:
    """MATLAB struct {Q, data, info} -> QSpace dict (labels int32)."""
    lib = _fake()
    Qc = lib.mxGetField(S, 0, b"Q")
    D = lib.mxGetField(S, 0, b"data")
    r = int(lib.mxGetNumberOfElements(Qc)) if Qc else 0
    n = int(lib.mxGetNumberOfElements(D)) if D else 0
    Q = [np.rint(_np_of(lib.mxGetCell(Qc, k))).astype(np.int32).reshape(n, -1) for k in range(r)]
    data = [_np_of(lib.mxGetCell(D, i)) for i in range(n)]
    info = {}
    I = lib.mxGetField(S, 0, b"info")
    if I and lib.mxIsStruct(I):
        t = lib.mxGetField(I, 0, b"itags")
        if t and lib.mxIsCell(t):
            info["itags"] = [_str_of(lib.mxGetCell(t, k)) for k in range(int(lib.mxGetNumberOfElements(t)))]
    return {"Q": Q, "data": data, "info": info}


def call(name: str, args: list, nout: int = 1) -> list:
    """Calls MEX `name` on mxArray arguments; returns the output mxArrays."""
    lib = _fake()
    fn = _mexfn(name)
    prhs = (C.c_void_p * len(args))(*args)
    plhs = (C.c_void_p * max(nout, 1))()
    rc = lib.fakemx_call(fn, name.encode(), nout, plhs, len(args), prhs)
    if rc:
        raise RefError(lib.fakemx_last_error().decode(errors="replace"))
    return [plhs[i] for i in range(nout)]


def _arg(x):
    if isinstance(x, str):
        return _mx_string(x)
    v = np.atleast_1d(np.asarray(x, dtype=np.float64)).reshape(1, -1)
    return _mx_array(v)


def contractQS(A: dict, ia, B: dict, ib, perm=None) -> dict:
    """The reference's contractQS(A, ia, B, ib [,perm])."""
    lib = _fake()
    args = [to_mx(A), _arg(ia), to_mx(B), _arg(ib)]
    if perm is not None:
        if isinstance(perm, str):  # '3,1,2' -> [3, 1, 2] (numeric perm argument)
            perm = [int(x) for x in perm.replace(",", " ").split()] if any(c in perm for c in ", ") \
                else [int(c) for c in perm]
        args.append(_arg(perm))
    try:
        out = call("contractQS", args, 1)[0]
        res = from_mx(out) if out else {"Q": [], "data": [], "info": {}}
        if out:
            lib.mxDestroyArray(out)
        return res
    finally:
        for a in args:
            lib.mxDestroyArray(a)


def contractQS_cell(items: list, perm=None) -> dict:
    """The reference's cell contraction contractQS({X0, X1, '*', ...} [,perm]):
    items are QSpace dicts or option strings ('*' after a QSpace)."""
    lib = _fake()
    cell = lib.mxCreateCellMatrix(1, len(items))
    for k, x in enumerate(items):
        lib.mxSetCell(cell, k, _mx_string(x) if isinstance(x, str) else to_mx(x))
    args = [cell]
    if perm is not None:
        args.append(_arg(perm))
    try:
        out = call("contractQS", args, 1)[0]
        res = from_mx(out) if out else {"Q": [], "data": [], "info": {}}
        if out:
            lib.mxDestroyArray(out)
        return res
    finally:
        for a in args:
            lib.mxDestroyArray(a)


def permuteQS(A: dict, perm, conj: bool = False) -> dict:
    """The reference's permuteQS(A, perm [,'conj'])."""
    lib = _fake()
    args = [to_mx(A), _arg(perm)]
    if conj:
        args.append(_mx_string("conj"))
    try:
        out = call("permuteQS", args, 1)[0]
        res = from_mx(out)
        lib.mxDestroyArray(out)
        return res
    finally:
        for a in args:
            lib.mxDestroyArray(a)


def plusQS(A: dict, B: dict, f: float = 1.0) -> dict:
    """The reference's plusQS(A, B [,f]) = A + f B."""
    lib = _fake()
    args = [to_mx(A), to_mx(B), _arg(float(f))]
    try:
        out = call("plusQS", args, 1)[0]
        res = from_mx(out) if out else {"Q": [], "data": [], "info": {}}
        if out:
            lib.mxDestroyArray(out)
        return res
    finally:
        for a in args:
            lib.mxDestroyArray(a)


def eigQS(H: dict, **opts) -> tuple:
    """The reference's [Etot, I] = eigQS(H, 'Nkeep', .., 'deps', .., 'Etrunc', ..):
    returns (Etot, {'AK','AD','EK','ED': QSpace dicts, 'NK': int})."""
    lib = _fake()
    args = [to_mx(H)]
    for k, v in opts.items():
        args += [_mx_string(k), _arg(v)]
    try:
        Etot, I = call("eigQS", args, 2)
        res = {k: from_mx(lib.mxGetField(I, 0, k.encode())) for k in ("AK", "AD", "EK", "ED")}
        res["NK"] = int(_np_of(lib.mxGetField(I, 0, b"NK")).ravel()[0])
        e = _np_of(Etot).copy()
        lib.mxDestroyArray(Etot)
        lib.mxDestroyArray(I)
        return e, res
    finally:
        for a in args:
            lib.mxDestroyArray(a)
