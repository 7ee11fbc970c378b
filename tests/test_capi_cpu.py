"""CPU-side checks: the C-ABI library loads and exports every symbol that
include/qsgpu.h declares; host-only entry points (markSet truncation) agree
with the oracle; errors are reported as status codes."""
import ctypes as C
import re
from pathlib import Path

import numpy as np
import pytest

from oracle import qs_oracle as orc
from qspace_gb300 import _capi

ROOT = Path(__file__).resolve().parents[1]


def header_symbols():
    txt = (ROOT / "include" / "qsgpu.h").read_text()
    return sorted(set(re.findall(r"^QS_EXPORT [^;(]*?\b(qs_[A-Za-z0-9_]+)\(", txt, flags=re.M)))


def test_library_exports_every_declared_symbol():
    lib = _capi.load()
    syms = header_symbols()
    assert len(syms) >= 25
    missing = [s for s in syms if not hasattr(lib, s)]
    assert not missing, missing
    # every declared symbol has a ctypes signature in the binding
    assert sorted(_capi.SIGNATURES) == syms


def test_version_and_error_text():
    lib = _capi.load()
    assert b"sm_103a" in lib.qs_version()


def test_ctx_without_gpu_is_a_status_not_a_crash():
    import torch
    if torch.cuda.is_available():
        pytest.skip("a GPU is present")
    lib = _capi.load()
    h = C.c_void_p()
    rc = lib.qs_ctx_create(0, C.byref(h))
    assert rc == 4  # QS_ERR_CUDA
    assert lib.qs_last_error()


def _mark(E_blocks, nkeep, etrunc, deps):
    lib = _capi.load()
    n = np.array([len(e) for e in E_blocks], np.int64)
    E = np.concatenate(E_blocks).astype(np.float64)
    keep = np.zeros(len(E), np.uint8)
    nk, et = C.c_int64(), C.c_double()
    rc = lib.qs_mark_keep(len(n), n.ctypes.data_as(_capi.c_int64_p), E.ctypes.data_as(_capi.c_double_p), None,
                          nkeep, etrunc, deps, keep.ctypes.data_as(C.POINTER(C.c_uint8)), C.byref(nk), C.byref(et))
    assert rc == 0
    return keep.astype(bool), nk.value


@pytest.mark.parametrize("nkeep,etrunc,deps", [(-1, 0, 0), (10, 0, 0), (50, 0, 0), (500, 0, 0),
                                               (200, 1.5, 0), (40, 0, 1e-12), (30, 0, 1e-3),
                                               (64, 0.8, 1e-6)])
def test_mark_keep_matches_oracle(nkeep, etrunc, deps):
    rng = np.random.default_rng(1)
    # blocks with degenerate multiplet-like levels
    E_blocks = []
    for b in range(12):
        base = np.sort(rng.uniform(-2, 3, size=int(rng.integers(1, 20))))
        E_blocks.append(np.repeat(base, int(rng.integers(1, 3))))
    k, nk = _mark(E_blocks, nkeep, etrunc, deps)
    ko, nko = orc.mark_keep(E_blocks, nkeep, etrunc, deps)
    assert nk == nko
    assert np.array_equal(k, np.concatenate(ko))


def test_mark_keep_rejects_weights():
    lib = _capi.load()
    n = np.array([2], np.int64)
    E = np.array([0.0, 1.0])
    w = np.array([1.0])
    keep = np.zeros(2, np.uint8)
    rc = lib.qs_mark_keep(1, n.ctypes.data_as(_capi.c_int64_p), E.ctypes.data_as(_capi.c_double_p),
                          w.ctypes.data_as(_capi.c_double_p), 1, 0.0, 0.0,
                          keep.ctypes.data_as(C.POINTER(C.c_uint8)), None, None)
    assert rc == 7


def test_index_parsing_matches_oracle():
    """The C++ planner and the oracle read index strings alike (checked
    through an error-free host-side parse: qs_mark_keep has no index, so
    compare the oracle on its own known answers)."""
    assert orc.parse_ctr_idx("12*") == ([0, 1], True)
    assert orc.parse_ctr_idx("1,3") == ([0, 2], False)
    assert orc.parse_ctr_idx("[2 3]**") == ([1, 2], False)
    assert orc.parse_ctr_idx("12,13") == ([11, 12], False)
    assert orc.parse_ctr_idx([2, 1]) == ([1, 0], False)
    with pytest.raises(ValueError):
        orc.parse_ctr_idx("1,1")
    with pytest.raises(ValueError):
        orc.parse_ctr_idx("0")
