"""Packing of QSpace dicts into .npz fixtures (no pickle)."""
from __future__ import annotations

import json

import numpy as np


def pack(prefix: str, A: dict, out: dict) -> None:
    n = len(A["data"])
    r = len(A["Q"])
    qd = int(np.asarray(A["Q"][0]).reshape(n, -1).shape[1]) if (r and n) else 0
    dims = np.array([(tuple(np.shape(d)) + (1,) * max(0, r - np.ndim(d)))[:r] for d in A["data"]],
                    np.int64).reshape(n, r)
    out[f"{prefix}_q"] = (np.stack([np.asarray(q).reshape(n, qd) for q in A["Q"]], axis=1).astype(np.int32)
                          if (r and n) else np.zeros((n, r, qd), np.int32))
    out[f"{prefix}_dims"] = dims
    cplx = any(np.iscomplexobj(d) for d in A["data"])
    flat = [np.asarray(d, np.complex128 if cplx else np.float64).reshape(-1, order="F") for d in A["data"]]
    out[f"{prefix}_data"] = np.concatenate(flat) if flat else np.zeros(0)
    out[f"{prefix}_meta"] = np.array(json.dumps({"rank": r, "nblk": n, "qdim": qd, "complex": cplx,
                                                 "itags": (A.get("info") or {}).get("itags")}))


def unpack(prefix: str, z) -> dict:
    meta = json.loads(str(z[f"{prefix}_meta"]))
    n, r = meta["nblk"], meta["rank"]
    q, dims, flat = z[f"{prefix}_q"], z[f"{prefix}_dims"], z[f"{prefix}_data"]
    Q = [np.ascontiguousarray(q[:, k, :]) for k in range(r)]
    data, o = [], 0
    for i in range(n):
        s = int(np.prod(dims[i])) if r else 1
        data.append(flat[o:o + s].reshape(tuple(dims[i]), order="F"))
        o += s
    info = {"itags": meta["itags"]} if meta.get("itags") else {}
    return {"Q": Q, "data": data, "info": info}
