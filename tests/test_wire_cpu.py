"""The QSpace wire container (qs_wire_size / qs_wire_pack / qs_wire_view):
every QSpace of the reference-generated fixtures survives pack -> view bit
for bit (labels, dims, block order, data, itags); views point into the
buffer without copying; malformed containers are refused with a status
before any pointer is formed.  Host-only entry points: no GPU needed."""
from pathlib import Path

import numpy as np
import pytest

from qspace_gb300 import QSpace
from qspace_gb300._capi import QSError
from qspace_gb300.qspace import from_wire, to_wire
from tests.golden.golden_io import unpack

G = Path(__file__).resolve().parent / "golden"
HDR = 128


def _fixture_qspaces():
    out = []
    for fname in ("contract_golden.npz", "permute_golden.npz", "cell_golden.npz"):
        z = np.load(G / fname)
        for k in z.keys():
            if k.endswith("_meta"):
                out.append((f"{fname}:{k[:-5]}", QSpace.from_dict(unpack(k[:-5], z))))
    return out


def _same(a: QSpace, b: QSpace):
    assert a.rank == b.rank and a.nblk == b.nblk
    assert a.info.get("itags") == b.info.get("itags")
    for k in range(a.rank if a.nblk else 0):
        assert np.array_equal(np.asarray(a.Q[k]).reshape(a.nblk, -1), np.asarray(b.Q[k]).reshape(b.nblk, -1))
    for x, y in zip(a.data, b.data):
        x, y = np.asarray(x), np.asarray(y)
        assert x.shape == y.shape or (x.size == y.size == 1)
        assert np.array_equal(x.reshape(-1).view(np.uint8), np.asarray(y, x.dtype).reshape(-1).view(np.uint8))


def _header(buf):
    h = np.frombuffer(buf, np.int64, 16, 0)
    return {"nblk": h[3], "nelem": h[4], "off_q": h[5], "off_dims": h[6], "off_offs": h[7],
            "off_data": h[8], "off_itags": h[9], "len_itags": h[10], "total": h[11]}


def test_fixture_round_trip_bit_exact():
    qs = _fixture_qspaces()
    assert len(qs) >= 100
    for name, A in qs:
        buf = to_wire(A)
        B = from_wire(buf)
        _same(A, B)
        h = _header(buf)
        assert h["total"] == buf.size and h["off_data"] % 64 == 0, name
        assert bytes(buf[:4]) == b"QSPW"


def test_view_is_zero_copy_and_read_only_from_bytes():
    rng = np.random.default_rng(1)
    A = QSpace([np.array([[0], [1]], np.int32), np.array([[0], [1]], np.int32)],
               [rng.standard_normal((3, 4)) + 1j * rng.standard_normal((3, 4)), rng.standard_normal((2, 5)) + 0j],
               {"itags": ["L", "R*"]})
    buf = to_wire(A)
    B = from_wire(buf)
    assert all(np.shares_memory(b, buf) for b in B.data)
    _same(A, B)
    Bb = from_wire(bytes(buf))                   # immutable source: read-only views
    assert not Bb.data[0].flags.writeable
    _same(A, Bb)


def test_empty_and_unlabelled():
    E = QSpace([np.zeros((0, 1), np.int32)] * 3, [], {})
    _same(E, from_wire(to_wire(E)))
    R = QSpace([np.array([[2, -1]], np.int32)], [np.arange(7.0)], {})
    _same(R, from_wire(to_wire(R)))


def _sample():
    A = QSpace([np.array([[0], [1], [2]], np.int32), np.array([[0], [1], [2]], np.int32)],
               [np.ones((2, 2)), np.full((1, 3), 2.0), np.full((4, 1), 3.0)], {"itags": ["a", "b*"]})
    return to_wire(A)


def _set64(b, byte_off, value):
    b[byte_off:byte_off + 8] = np.array([value], np.int64).view(np.uint8)
    return b


def _code(buf):
    with pytest.raises(QSError) as e:
        from_wire(buf)
    return e.value.code


def test_malformed_containers_are_refused():
    good = _sample()
    h = _header(good)
    assert _code(good[:HDR - 1]) == 1                         # shorter than the header
    assert _code(good[:int(h["total"]) - 1]) == 1             # truncated
    b = good.copy(); b[0] = ord("X"); assert _code(b) == 1    # magic
    b = good.copy(); b[4] = 2; assert _code(b) == 7           # format version
    b = good.copy(); b[8] = 4; assert _code(b) == 1           # unknown flag
    b = good.copy(); b[20:24] = 0; assert _code(b) == 1       # byte-order mark
    assert _code(_set64(good.copy(), 64, h["off_data"] + 8)) == 1    # data section misaligned
    assert _code(_set64(good.copy(), 40, h["off_dims"])) == 1        # sections overlap
    assert _code(_set64(good.copy(), 88, 1 << 40)) == 1              # total beyond the buffer
    b = good.copy(); b[int(h["off_itags"] + h["len_itags"]) - 1] = ord("x"); assert _code(b) == 1  # no NUL
    # a block reaching past the data section
    assert _code(_set64(good.copy(), int(h["off_dims"]), 50)) == 2
    # a negative offset
    assert _code(_set64(good.copy(), int(h["off_offs"]) + 8, -4)) == 2
    # the untouched container still reads
    assert from_wire(good).nblk == 3


def test_misaligned_source_is_copied():
    good = _sample()
    raw = bytearray(good.size + 1)
    raw[1:] = good.tobytes()
    B = from_wire(memoryview(raw)[1:])
    assert B.nblk == 3 and B.info["itags"] == ["a", "b*"]
