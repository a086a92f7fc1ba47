"""GROUP BY a small-range key with f64 arguments (the one-pass small-key form) through the C ABI.

Counts, first rows, MIN and MAX are exact; SUM and AVG within 1e-12 relative of the exactly rounded sum
(math.fsum), whatever the values' signs and magnitudes; NaN and infinite values give the IEEE sums (NaN,
+inf, -inf, and NaN for +inf with -inf) and are left out of MIN and MAX. Keys of 5, 50 and 64 values (the
form's limit), eight distinct columns, and columns with an infinite zone range or none.
"""
import math

import numpy as np
import pytest

pytestmark = pytest.mark.gpu
COUNT, SUM, AVG, MIN, MAX = 0, 1, 2, 3, 4


@pytest.fixture(scope="module")
def ops(gpu):
    from computeql_gb300 import ops as o
    return o


def column(ops, arr):
    """a device column whose zone range skips NaN and infinities, as a zone map does"""
    fin = arr[np.isfinite(arr)] if arr.dtype.kind == "f" else arr
    zone = (float(fin.min()), float(fin.max())) if len(fin) else None
    return ops.Column(ops.TYPE_F64 if arr.dtype == np.float64 else ops.TYPE_F32 if arr.dtype == np.float32 else
                      ops.TYPE_I32 if arr.dtype == np.int32 else ops.TYPE_U32, len(arr), ops.DeviceBuffer(arr.nbytes, arr), zone=zone)


def ieee_sum(x):
    x = np.asarray(x, dtype=np.float64)
    if np.isnan(x).any() or (np.isposinf(x).any() and np.isneginf(x).any()):
        return math.nan
    if np.isposinf(x).any():
        return math.inf
    if np.isneginf(x).any():
        return -math.inf
    return math.fsum(x)


def check(res, key, funcs, args, first_key):
    present = np.unique(key)
    assert res["groups"] == len(present)
    for g, k in enumerate(present):
        m = key == k
        assert res["repr_row"][g] == np.argmax(m)
        assert res["counts"][g] == m.sum()
        for e, (f, a) in enumerate(zip(funcs, args)):
            got = res["results"][g, e]
            if f == COUNT:
                assert got == m.sum()
                continue
            x = a[m].astype(np.float64)
            if f in (SUM, AVG):
                want = ieee_sum(x)
                if f == AVG:
                    want = want / m.sum()
                if math.isnan(want) or math.isinf(want):
                    assert (math.isnan(got) and math.isnan(want)) or got == want
                else:
                    floor = 1.0 if f == SUM else 1.0 / m.sum()
                    assert abs(got - want) <= 1e-12 * max(abs(want), floor), (k, f, got, want)
            else:
                fin = x[~np.isnan(x)]
                want = (fin.min() if f == MIN else fin.max()) if len(fin) else (1.0e300 if f == MIN else -1.0e300)
                assert got == want or (got == 0.0 and want == 0.0)


@pytest.mark.parametrize("values", [5, 50, 64])
def test_lognormal_and_mixed_sign_measures(ops, values):
    rng = np.random.default_rng(values)
    n = 2_000_003
    key = (rng.integers(0, values, n) + 7).astype(np.uint32)
    key[0], key[1] = 7, 7 + values - 1           # the whole range present
    logn = np.exp(3.0 + rng.normal(size=n))
    mixed = rng.normal(size=n) * 10.0 ** rng.integers(-3, 6, n)
    mixed[::1000] = -0.0
    f32 = rng.normal(size=n).astype(np.float32)
    i32 = rng.integers(-2**31, 2**31 - 1, n).astype(np.int32)
    kc = ops.Column.from_numpy(key)
    cols = [column(ops, a) for a in (logn, mixed, f32, i32)]
    funcs = [COUNT, SUM, AVG, MIN, MAX, AVG, SUM, MAX]
    args = [None, logn, mixed, mixed, logn, f32, i32, i32]
    dev = [None, cols[0], cols[1], cols[1], cols[0], cols[2], cols[3], cols[3]]
    res = ops.group_hash([kc], funcs, dev)
    assert res["path"] == 3
    check(res, key, funcs, args, 7)


def test_nan_and_infinities(ops):
    rng = np.random.default_rng(3)
    n = 500_000
    key = rng.integers(0, 6, n).astype(np.uint32)
    x = rng.normal(size=n) * 1e3
    x[key == 1] = np.where(rng.random((key == 1).sum()) < 0.01, np.nan, x[key == 1])
    sel2 = np.flatnonzero(key == 2)
    x[sel2[::5000]] = np.inf
    sel3 = np.flatnonzero(key == 3)
    x[sel3[::7000]] = -np.inf
    sel4 = np.flatnonzero(key == 4)
    x[sel4[0]], x[sel4[1]] = np.inf, -np.inf
    x[key == 5] = np.nan                          # every value NaN: MIN and MAX keep their starting values
    funcs = [COUNT, SUM, AVG, MIN, MAX]
    args = [None, x, x, x, x]
    xc = column(ops, x)
    res = ops.group_hash([ops.Column.from_numpy(key)], funcs, [None, xc, xc, xc, xc])
    assert res["path"] == 3
    check(res, key, funcs, args, 0)


def test_eight_measures_with_cancelling_sums(ops):
    # eight distinct columns of mixed-sign values whose group sums cancel to far below their terms
    rng = np.random.default_rng(11)
    n = 300_000
    key = rng.integers(0, 9, n).astype(np.uint32)
    arrs = [rng.normal(size=n) * (i + 1) for i in range(8)]
    cols = [column(ops, a) for a in arrs]
    funcs = [SUM] * 8
    res = ops.group_hash([ops.Column.from_numpy(key)], funcs, cols)
    assert res["path"] == 3
    check(res, key, funcs, arrs, 0)


@pytest.mark.parametrize("zone", ["infinite", "none"])
def test_column_without_a_finite_range(ops, zone):
    # a summed f64 column whose zone range is infinite, or that has none: its scale comes from a pass that
    # finds its largest finite magnitude
    rng = np.random.default_rng(12)
    n = 300_000
    key = rng.integers(0, 9, n).astype(np.uint32)
    x = np.exp(rng.normal(size=n))
    x[np.flatnonzero(key == 4)[3]] = np.inf
    xc = ops.Column.from_numpy(x)
    assert xc.zone[1] == np.inf
    if zone == "none":
        xc = ops.Column(ops.TYPE_F64, n, xc.buffer, zone=None)
    funcs = [COUNT, SUM, AVG]
    res = ops.group_hash([ops.Column.from_numpy(key)], funcs, [None, xc, xc])
    assert res["path"] == 3
    check(res, key, funcs, [None, x, x], 0)


@pytest.mark.parametrize("seed", range(6))
def test_random_shapes(ops, seed):
    # random key ranges (1 to 64 values, negative keys too), column types and aggregate mixes
    rng = np.random.default_rng(100 + seed)
    n = int(rng.integers(1, 400_000))
    values = int(rng.integers(1, 65))
    low = int(rng.integers(-1000, 1000))
    key = (rng.integers(0, values, n) + low).astype(np.int32)
    cols, arrs = [], []
    for c in range(int(rng.integers(1, 5))):
        kind = rng.integers(0, 4)
        if kind == 0:
            a = rng.normal(size=n) * 10.0 ** int(rng.integers(-5, 8))
        elif kind == 1:
            a = (rng.normal(size=n) * 1000).astype(np.float32)
        elif kind == 2:
            a = rng.integers(-2**31, 2**31 - 1, n).astype(np.int32)
        else:
            a = rng.integers(0, 2**31 - 1, n).astype(np.uint32)
        arrs.append(a)
        cols.append(column(ops, a))
    funcs, args, dev = [], [], []
    for e in range(int(rng.integers(1, 9))):
        f = int(rng.integers(0, 5))
        c = int(rng.integers(0, len(cols)))
        funcs.append(f)
        args.append(None if f == COUNT else arrs[c])
        dev.append(None if f == COUNT else cols[c])
    if all(f == COUNT for f in funcs) or all(a is None or a.dtype.kind != "f" for a in args):
        funcs.append(SUM)                      # one f32/f64 argument makes it this path's
        fa = next((i for i, a in enumerate(arrs) if a.dtype.kind == "f"), None)
        if fa is None:
            arrs.append(rng.normal(size=n))
            cols.append(column(ops, arrs[-1]))
            fa = len(arrs) - 1
        args.append(arrs[fa])
        dev.append(cols[fa])
        funcs, args, dev = funcs[-8:], args[-8:], dev[-8:]
    res = ops.group_hash([ops.Column.from_numpy(key)], funcs, dev)
    assert res["path"] == 3
    check(res, key, funcs, args, low)
