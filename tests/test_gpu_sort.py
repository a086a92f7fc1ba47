"""ORDER BY through the C ABI (cqlops_sort_rows) against the oracle, row for row.

The oracle orders rows as the reference does (keys compared as F64, DESC per key, ties by input
position), so the GPU permutation must equal it exactly, not just be "a" valid order. Cases: every
ORDER BY of the reference's sort test (src/tests/bench_query_sort.c:256-268) on its table at the test's
default 3M rows, plain and --narrow; each key type with negatives, -0.0 and infinities; narrow and
sequence encodings; tile edges; a filtered row set (ORDER BY an f64 measure over a 200k-row subset of a
10M-row table); and the reference's own property check at 100M rows.
"""
import numpy as np
import pytest

import oracle
from tests.sort_table import SORT_CASES, pq_table, verify_order

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def ops(gpu):
    from computeql_gb300 import ops as o
    return o


@pytest.fixture(scope="module")
def pq(ops):
    tables = {}
    for narrow in (False, True):
        t = pq_table(3000000, narrow)
        cols = {c: ops.Column.from_numpy(t[c]) for c in "abcde"}
        tables[narrow] = (t, cols)
    return tables


@pytest.mark.parametrize("narrow", [False, True])
@pytest.mark.parametrize("case", range(len(SORT_CASES)))
def test_reference_sort_cases(ops, pq, case, narrow):
    t, cols = pq[narrow]
    keys = SORT_CASES[case]
    got = ops.sort_rows([cols[c] for c, _ in keys], [d for _, d in keys])
    want = oracle.sort_rows([t[c] for c, _ in keys], [d for _, d in keys])
    assert verify_order(t, keys, got) == 0
    assert np.array_equal(got, want)


def _typed(dtype, n, rng):
    if dtype == np.float64:
        v = rng.normal(0, 1e3, n)
        v[::97] = -0.0
        v[1::97] = 0.0
        v[::1001] = np.inf
        v[3::1001] = -np.inf
        v[5::13] = 12.5                                    # ties, broken by row id
        return v
    if dtype == np.float32:
        return _typed(np.float64, n, rng).astype(np.float32)
    if dtype == np.int64:
        v = rng.integers(-2**62, 2**62, n)
        v[::7] = 2**53 + rng.integers(0, 4, len(v[::7]))   # values that meet in F64
        return v.astype(np.int64)
    if dtype == np.uint64:
        return rng.integers(0, 2**64 - 1, n, dtype=np.uint64, endpoint=True)
    info = np.iinfo(dtype)
    return rng.integers(info.min, info.max, n, endpoint=True).astype(dtype)


@pytest.mark.parametrize("desc", [0, 1])
@pytest.mark.parametrize("dtype", [np.uint32, np.int32, np.float32, np.float64, np.uint64, np.int64])
def test_single_key_types(ops, dtype, desc):
    rng = np.random.default_rng(21)
    v = _typed(dtype, 300001, rng)
    got = ops.sort_rows([ops.Column.from_numpy(v)], [desc])
    assert np.array_equal(got, oracle.sort_rows([v], [desc]))


@pytest.mark.parametrize("n", [0, 1, 2, 4095, 4096, 4097, 8192 + 31])
def test_tile_edges(ops, n):
    rng = np.random.default_rng(n)
    a = rng.integers(0, 7, n).astype(np.uint32)
    b = rng.normal(size=n)
    if n == 0:
        got = ops.sort_rows([ops.Column(ops.TYPE_U32, 0, ops.DeviceBuffer(16))])
        assert len(got) == 0
        return
    got = ops.sort_rows([ops.Column.from_numpy(a), ops.Column.from_numpy(b)], [1, 0])
    assert np.array_equal(got, oracle.sort_rows([a, b], [1, 0]))


def test_narrow_and_sequence_keys(ops):
    rng = np.random.default_rng(5)
    n = 500000
    small = rng.integers(-100, 100, n).astype(np.int32)     # u8 codes
    mid = rng.integers(7, 40000, n).astype(np.uint32)        # u16 codes
    c_small = ops.Column.from_numpy(small, narrow=True)
    c_mid = ops.Column.from_numpy(mid, narrow=True)
    assert c_small.width == 1 and c_mid.width == 2
    seq = ops.Column.sequence(n, first=1000)
    got = ops.sort_rows([c_small, c_mid, seq], [0, 1, 1])
    ids = np.arange(1000, 1000 + n, dtype=np.uint32)
    assert np.array_equal(got, oracle.sort_rows([small, mid, ids], [0, 1, 1]))


def test_all_equal_keys_keep_input_order(ops):
    v = np.full(100000, 3.5)
    assert np.array_equal(ops.sort_rows([ops.Column.from_numpy(v)], [1]), np.arange(100000))


@pytest.mark.parametrize("desc", [0, 1])
def test_passes_whose_digit_does_not_vary(ops, desc):
    # u32 keys below 2^24 (the high byte's pass is a copy), whole-number f64 keys (the low mantissa bytes'
    # passes are copies), and both under a row selection, whose last pass maps positions to its rows
    rng = np.random.default_rng(31 + desc)
    n = 300001
    small = rng.integers(0, 1 << 24, n).astype(np.uint32)
    whole = rng.integers(-5000, 5000, n).astype(np.float64)
    for v in (small, whole):
        got = ops.sort_rows([ops.Column.from_numpy(v)], [desc])
        assert np.array_equal(got, oracle.sort_rows([v], [desc]))
    sel = np.sort(rng.choice(n, 70001, replace=False)).astype(np.uint32)
    buf = ops.DeviceBuffer(sel.nbytes, sel)
    got = ops.sort_rows([ops.Column.from_numpy(whole), ops.Column.from_numpy(small)], [desc, 0], selection=buf)
    want = sel[oracle.sort_rows([whole[sel], small[sel]], [desc, 0])]
    assert np.array_equal(got, want)


def test_filtered_subset_f64_measure(ops):
    # a 10M-row table with a lognormal f64 measure; ORDER BY it over the ~200k rows a filter keeps
    rng = np.random.default_rng(9)
    n = 10_000_000
    measure = np.round(rng.lognormal(3.0, 1.0, n), 2)   # rounded: many ties, broken by row id
    status = rng.integers(0, 50, n).astype(np.uint32)
    rows = np.nonzero(status == 17)[0].astype(np.uint32)
    sel = ops.DeviceBuffer(rows.nbytes, rows)
    got = ops.sort_rows([ops.Column.from_numpy(measure)], [0], selection=sel)
    want = rows[oracle.sort_rows([measure[rows]], [0])]
    assert len(got) == len(rows)
    assert np.array_equal(got, want)
    got_desc = ops.sort_rows([ops.Column.from_numpy(measure), ops.Column.from_numpy(status)], [1, 0], selection=sel)
    assert np.array_equal(got_desc, rows[oracle.sort_rows([measure[rows], status[rows]], [1, 0])])


def test_property_check_100m(ops):
    # the reference's own check (permutation, keys in order, ties by position) at 100M rows
    n = 100_000_000
    col = ops.Column.splitmix(n, 0, 4, 1, 10000)
    got = ops.sort_rows([col], [1])
    v = col.buffer.read(np.uint32)
    assert len(got) == n
    assert np.bincount(got, minlength=n).max() == 1
    sv = v[got]
    assert np.all(sv[:-1] >= sv[1:])
    tie = sv[:-1] == sv[1:]
    assert np.all(got[:-1][tie] < got[1:][tie])
