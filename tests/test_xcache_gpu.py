"""Device-resident CG / X-symbol factor table (qs_xcache_*) and the keyed
grouped product (qs_grouped_gemm_keyed): lookups agree with a host dict
(inserts, overwrites, missing keys), the reserved key and a full table are
refused without changing the table, a table may outlive its context, and a
keyed product equals, bit for bit,
the same product with the factors passed in the pair list (plain FP64 and
split paths, real and complex; shared keys as X-symbols are shared between
pairs; a changed factor is seen by the next call; a missing key is an
error)."""
import numpy as np
import pytest

torch = pytest.importorskip("torch")

from qspace_gb300._capi import QSError
from qspace_gb300.grouped import DeviceBatch, FactorTable, Packed
from qspace_gb300.workloads import grouped_pairs

pytestmark = pytest.mark.gpu


def _zero(db):
    # torch's stream and the library's stream are not ordered with each other
    db.dC.zero_()
    torch.cuda.synchronize()


def _out(db):
    db.ctx.sync()
    return db.dC.cpu().numpy()


def _keys(rng, n):
    return rng.integers(0, 2 ** 63, size=(n, 2), dtype=np.uint64) * np.uint64(2) + np.uint64(1)


def test_put_get_matches_dict(ctx):
    rng = np.random.default_rng(1)
    T = FactorTable(20000, ctx)
    ref = {}
    k1, v1 = _keys(rng, 6000), rng.standard_normal(6000)
    T.put(k1, v1)
    ref.update({tuple(k): v for k, v in zip(k1.tolist(), v1)})
    # overwrite half, add new ones, include small keys and a zero word
    k2 = np.concatenate([k1[::2], _keys(rng, 3000), np.array([[0, 0], [0, 7], [5, 0]], np.uint64)])
    v2 = rng.standard_normal(len(k2))
    T.put(k2, v2)
    ref.update({tuple(k): v for k, v in zip(k2.tolist(), v2)})
    assert len(T) == len(ref)
    missing = _keys(rng, 1000)
    q = np.concatenate([np.array(list(ref.keys()), np.uint64), missing])
    vals, found = T.get(q)
    n = len(ref)
    assert found[:n].all() and not found[n:].any()
    assert np.array_equal(vals[:n], np.array(list(ref.values())))
    assert np.all(vals[n:] == 0.0)
    T.close()


def test_reserved_key_and_full_table(ctx):
    rng = np.random.default_rng(2)
    T = FactorTable(100, ctx)
    top = np.uint64(2 ** 64 - 1)
    with pytest.raises(QSError) as e:
        T.put(np.array([[top, top]], np.uint64), [1.0])
    assert e.value.code == 1
    k = _keys(rng, 100)
    T.put(k, np.arange(100.0))
    cap_keys = _keys(rng, 200)
    with pytest.raises(QSError) as e:
        T.put(cap_keys, np.ones(200))
    assert e.value.code == 5
    assert len(T) == 100                      # the refused batch changed nothing
    vals, found = T.get(k)
    assert found.all() and np.array_equal(vals, np.arange(100.0))
    assert not T.get(cap_keys)[1].any()
    T.close()


@pytest.mark.parametrize("cplx", [False, True])
@pytest.mark.parametrize("prec", ["fp64", "split"])
def test_keyed_product_equals_listed_factors(ctx, cplx, prec):
    rng = np.random.default_rng(3)
    w = grouped_pairs(seed=7, npairs=60, lo=4, hi=200, complex_data=cplx)
    n = len(w["M"])
    pool = _keys(rng, 12)                     # factors shared between pairs
    pool_vals = rng.uniform(-1.5, 1.5, 12)
    pool_vals[3] = 1.0                        # factor 1 and an exact zero
    pool_vals[7] = 0.0
    which = rng.integers(0, 12, n)
    fkeys = pool[which]
    T = FactorTable(64, ctx)
    T.put(pool, pool_vals)

    def listed(vals):
        db = DeviceBatch(Packed(w["A"], w["B"], vals[which], cplx=cplx), ctx)
        _zero(db)
        db.run(prec)
        return _out(db)

    db = DeviceBatch(Packed(w["A"], w["B"], np.full(n, 123.0), cplx=cplx), ctx)   # listed factors ignored
    _zero(db)
    db.run_keyed(fkeys, T, prec)
    got = _out(db)
    assert np.any(got != 0) and np.array_equal(got, listed(pool_vals))
    # a changed factor is seen by the next call, without new keys
    pool_vals[5] = -0.375
    T.put(pool[5:6], pool_vals[5:6])
    _zero(db)
    db.run_keyed(fkeys, T, prec)
    assert np.array_equal(_out(db), listed(pool_vals))
    T.close()


def test_missing_key_fails(ctx):
    rng = np.random.default_rng(4)
    w = grouped_pairs(seed=8, npairs=10, lo=4, hi=64, complex_data=False)
    T = FactorTable(16, ctx)
    keys = _keys(rng, 10)
    T.put(keys[:9], np.ones(9))
    db = DeviceBatch(Packed(w["A"], w["B"], np.ones(10), cplx=False), ctx)
    for prec in ("fp64", "split"):
        with pytest.raises(QSError) as e:
            db.run_keyed(keys, T, prec)
        assert e.value.code == 1
    # the context stays usable
    T.put(keys[9:], [2.0])
    db.run_keyed(keys, T, "fp64")
    T.close()


def test_table_outlives_its_context():
    """A table whose context is destroyed first is refused, then destroyed
    without touching the freed context."""
    from qspace_gb300.qspace import Context
    c2 = Context(0)
    T = FactorTable(16, c2)
    T.put(np.array([[1, 2]], np.uint64), [0.5])
    c2.close()
    with pytest.raises(QSError) as e:
        T.put(np.array([[3, 4]], np.uint64), [1.0])
    assert e.value.code == 1
    T.close()
