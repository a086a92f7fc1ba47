"""scan_simple through the C ABI against the oracle (counts and row sets bit-exact)."""
import json
import os

import numpy as np
import pytest

import oracle
from tests import closed_form as cf

pytestmark = pytest.mark.gpu
GOLDEN = os.path.join(os.path.dirname(__file__), "golden")
EQ, LT, LE, GT, GE = 0, 1, 2, 3, 4


@pytest.fixture(scope="module")
def ops(gpu):
    from computeql_gb300 import ops as o
    return o


def test_c1_count_flag_lt_2_matches_golden(ops):
    from computeql_gb300 import workloads
    fx = json.load(open(os.path.join(GOLDEN, "c1_oracle.json")))
    t = workloads.fact_table(fx["rows"])
    cnt, _ = ops.scan_simple([t.flag], [(0, LT, 2)])
    assert cnt == fx["count_flag_lt_2"]


@pytest.mark.parametrize("n", [1, 7, 8, 9, 10001, 1000003, 5_000_000])
def test_closed_form_filters(ops, n):
    idc, region, amount, _ = oracle.closed_form(n)
    exp = cf.expected(n)
    a = ops.Column.from_numpy(amount)
    r = ops.Column.from_numpy(region)
    assert ops.scan_simple([a], [(0, GT, cf.HIGH_AMOUNT)])[0] == exp["count_amount_gt_9990"]
    assert ops.scan_simple([r], [(0, EQ, 7)])[0] == exp["count_region_eq_7"]
    # id is its row number plus one: stored, and as a sequence the kernel computes
    for idcol in (ops.Column.from_numpy(idc), ops.Column.sequence(n, 1)):
        assert ops.scan_simple([idcol], [(0, GT, 1000), (0, LE, 900000000)])[0] == exp["count_id_range"]
    # narrow encodings of the same columns
    an = ops.Column.from_numpy(amount, narrow=True)
    rn = ops.Column.from_numpy(region, narrow=True)
    assert ops.scan_simple([an], [(0, GT, cf.HIGH_AMOUNT)])[0] == exp["count_amount_gt_9990"]
    assert ops.scan_simple([rn], [(0, EQ, 7)])[0] == exp["count_region_eq_7"]
    zc, zrows = ops.scan_simple([rn], [(0, GE, 20), (0, LE, 29)], want_rows=True)
    assert [zc, float(amount[zrows].astype(np.float64).sum())] == list(exp["join_zone2"])


def _column(dtype, n, rng):
    if dtype == np.uint32:
        return rng.integers(0, 1000, n).astype(np.uint32)
    if dtype == np.int32:
        return rng.integers(-500, 500, n).astype(np.int32)
    if dtype == np.float32:
        return (rng.integers(-500, 500, n) / 4.0).astype(np.float32)
    return (rng.integers(-500, 500, n) / 8.0).astype(np.float64)


@pytest.mark.parametrize("dtype", [np.uint32, np.int32, np.float32, np.float64])
@pytest.mark.parametrize("op", [EQ, LT, LE, GT, GE])
@pytest.mark.parametrize("target", [-3.5, 0.0, 17.0, 17.25, 499.0, 1e12, -1e12, float("nan")])
def test_single_leaf_matches_oracle(ops, dtype, op, target):
    n = 20011
    rng = np.random.default_rng(abs(hash((str(dtype), op))) % 1000)
    a = _column(dtype, n, rng)
    cnt, rows = ops.scan_simple([ops.Column.from_numpy(a)], [(0, op, target)], want_rows=True)
    ecnt, erows = oracle.scan_and([(a, op, target)], n, want_rows=True)
    assert cnt == ecnt
    assert np.array_equal(rows, erows)


@pytest.mark.parametrize("n", [1, 2, 7, 8, 9, 15, 16, 17, 255, 256, 2047, 2048, 2049, 100000])
def test_ragged_sizes_and_multi_leaf(ops, n):
    rng = np.random.default_rng(n)
    cols = [_column(np.uint32, n, rng), _column(np.int32, n, rng), _column(np.float64, n, rng), _column(np.float32, n, rng)]
    leaves = [(0, GE, 100), (1, LT, 300), (2, GT, -40.0), (3, LE, 100.0), (0, LT, 950), (1, GE, -480)]
    dev = [ops.Column.from_numpy(c) for c in cols]
    cnt, rows = ops.scan_simple(dev, leaves, want_rows=True)
    ecnt, erows = oracle.scan_and([(cols[c], op, t) for c, op, t in leaves], n, want_rows=True)
    assert cnt == ecnt
    assert np.array_equal(rows, erows)


def test_eight_leaves_narrow_and_wide_mix(ops):
    n = 333_333
    rng = np.random.default_rng(5)
    a = rng.integers(1000, 1200, n).astype(np.uint32)
    b = rng.integers(-30000, 30000, n).astype(np.int32)
    cols = [ops.Column.from_numpy(a, narrow=True), ops.Column.from_numpy(b, narrow=True), ops.Column.from_numpy(a), ops.Column.from_numpy(b)]
    assert cols[0].width == 1 and cols[1].width == 2
    leaves = [(0, GE, 1010), (1, LT, 20000), (2, LE, 1190), (3, GT, -25000), (0, LT, 1195.5), (1, GE, -29999.5), (2, GT, 1011), (3, LE, 19999)]
    cnt, rows = ops.scan_simple(cols, leaves, want_rows=True)
    srcs = [a, b, a, b]
    ecnt, erows = oracle.scan_and([(srcs[c], op, t) for c, op, t in leaves], n, want_rows=True)
    assert cnt == ecnt
    assert np.array_equal(rows, erows)


def test_output_grows_when_over_the_default_cap(ops):
    # 50 % selective: more than the max(65536, rows/32) first guess, so the second attempt runs
    n = 1_000_000
    a = np.arange(n, dtype=np.uint32) % 2
    cnt, rows = ops.scan_simple([ops.Column.from_numpy(a)], [(0, EQ, 1)], want_rows=True)
    assert cnt == n // 2
    assert np.array_equal(rows, np.arange(1, n, 2, dtype=np.uint32))


def test_no_match_and_all_match(ops):
    n = 100_000
    a = np.full(n, 5, dtype=np.uint32)
    col = ops.Column.from_numpy(a)
    assert ops.scan_simple([col], [(0, EQ, 6)])[0] == 0
    assert ops.scan_simple([col], [(0, EQ, 5)])[0] == n
    assert ops.scan_simple([col], [(0, LT, -1)])[0] == 0


# ---- zone maps and zone-map pruning (cql_zone_map, cqlops_scan_ranges) ----

@pytest.mark.parametrize("dtype,narrow", [(np.uint32, False), (np.int32, True), (np.uint32, True), (np.float32, False), (np.float64, False)])
def test_zone_map_matches_numpy(ops, dtype, narrow):
    rng = np.random.default_rng(3)
    n = 8192 * 37 + 1234
    if dtype == np.float64:
        v = rng.normal(size=n)
        v[8192 * 3: 8192 * 4] = np.nan               # a chunk with no values
        v[5] = np.nan
    elif dtype == np.float32:
        v = rng.normal(size=n).astype(np.float32)
    else:
        v = (rng.integers(-100, 100, n) if dtype == np.int32 else rng.integers(0, 60000 if narrow else 2**32, n)).astype(dtype)
    c = ops.Column.from_numpy(v, narrow=narrow)
    if narrow:
        assert c.width in (1, 2)
    zm = c.zone_map.reshape(-1, 2)[:-1]
    summary = c.zone_map[-2:]
    has = zm[:, 0] <= zm[:, 1]
    assert (summary[0], summary[1]) == (zm[has, 0].max(), zm[has, 1].min())
    for z in range(len(zm)):
        part = v[z * 8192:(z + 1) * 8192].astype(np.float64)
        part = part[~np.isnan(part)]
        if len(part) == 0:
            assert zm[z, 0] > zm[z, 1]
        else:
            assert (zm[z, 0], zm[z, 1]) == (part.min(), part.max())


@pytest.mark.parametrize("n", [1_000_000_007, 30_000_000])
def test_point_lookup_on_sequence_scans_one_chunk(ops, n):
    ids = ops.Column.sequence(n, 0)
    for k in (0, 8191, 8192, n // 3, n - 1, n + 5):
        cnt, rows = ops.scan_simple([ids], [(0, EQ, k)], want_rows=True, max_rows=16)
        assert cnt == (1 if k < n else 0)
        assert list(rows) == ([k] if k < n else [])
    cnt, rows = ops.scan_simple([ids], [(0, GE, n - 20000), (0, LT, n - 100)], want_rows=True)
    assert cnt == 19900 and np.array_equal(rows, np.arange(n - 20000, n - 100, dtype=np.uint32))


def test_pruning_on_a_clustered_column(ops):
    # a column sorted in blocks: zone maps prune most chunks; results equal the unpruned oracle
    rng = np.random.default_rng(7)
    n = 50_000_000
    ts = np.sort(rng.integers(0, 10**9, n)).astype(np.uint32)
    val = rng.integers(0, 100, n).astype(np.uint32)
    tcol, vcol = ops.Column.from_numpy(ts), ops.Column.from_numpy(val)
    for lo, hi in [(10**8, 10**8 + 10**6), (5 * 10**8, 6 * 10**8), (0, 3000)]:
        leaves = [(0, GE, lo), (0, LT, hi), (1, LT, 30)]
        cnt, rows = ops.scan_simple([tcol, vcol], leaves, want_rows=True)
        m = (ts >= lo) & (ts < hi) & (val < 30)
        assert cnt == m.sum()
        assert np.array_equal(rows, np.nonzero(m)[0].astype(np.uint32))
    # many scattered hits: the skip-bitmap form
    ts2 = ts.copy()
    ts2[::400_000] = 7
    c2 = ops.Column.from_numpy(ts2)
    cnt, rows = ops.scan_simple([c2], [(0, LE, 7)], want_rows=True)
    m = ts2 <= 7
    assert cnt == m.sum() and np.array_equal(rows, np.nonzero(m)[0].astype(np.uint32))


@pytest.mark.parametrize("case", ["random", "clustered", "none", "small_buffer"])
def test_selection_kept_on_the_device(ops, case):
    # scan_select lists the matching rows into a device buffer in the scan's own batch: the same rows, in the
    # same order, as scan_simple's host list; a zone-pruned scan, one with no match, and a buffer smaller than
    # the match count (the first rows, and the full count)
    rng = np.random.default_rng(17)
    n = 2_000_003
    if case == "clustered":
        v = np.sort(rng.integers(0, 1_000_000, n)).astype(np.uint32)
        leaves = [(0, GE, 400_000), (0, LT, 400_900)]
    else:
        v = rng.integers(0, 1_000_000, n).astype(np.uint32)
        leaves = [(0, GT, 2_000_000)] if case == "none" else [(0, LT, 30_000)]
    col = ops.Column.from_numpy(v)
    want_count, want_rows = ops.scan_simple([col], leaves, want_rows=True)
    cap = max(want_count // 3, 1) if case == "small_buffer" else n
    out = ops.DeviceBuffer(cap * 4)
    count = ops.scan_select([col], leaves, out)
    assert count == want_count
    m = min(count, cap)
    assert np.array_equal(out.read(np.uint32, m), want_rows[:m])
    if case == "clustered":
        # the selection feeds an operator that takes one: ORDER BY the values over the selected rows
        got = ops.sort_rows([col], [1], selection=out, count=count)
        assert np.array_equal(got, want_rows[oracle.sort_rows([v[want_rows]], [1])])
