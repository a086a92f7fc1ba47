"""ROW_NUMBER / RANK / DENSE_RANK on the GPU (cqlops_window_rank) against the oracle, row for row, on the
reference's window-rank test table and cases (bench_query_window_rank.c), plus integer, narrow and
sequence keys, a selection, one row and none."""
import numpy as np
import pytest

import oracle
from tests.window_table import CASES, tables, verify

pytestmark = pytest.mark.gpu

N = 200_003


@pytest.fixture(scope="module")
def ops(gpu):
    from computeql_gb300 import ops as o
    return o


@pytest.fixture(scope="module")
def table():
    return tables(N)


def _same(got, want):
    rows, rn, rk, dr = want
    assert np.array_equal(got["rows"], rows.astype(np.uint32))
    assert np.array_equal(got["row_number"], rn)
    assert np.array_equal(got["rank"], rk)
    assert np.array_equal(got["dense_rank"], dr)


@pytest.mark.parametrize("case", CASES, ids=[c[0] for c in CASES])
def test_reference_cases(ops, table, case):
    label, nk, parts, mask, narrow = case
    wide, nar = table
    keys = (nar if narrow else wide)[:nk]
    desc = [(mask >> k) & 1 for k in range(nk)]
    cols = [ops.Column.from_numpy(k) for k in keys]
    got = ops.window_rank(cols, desc, parts)
    assert verify(keys, desc, parts, got["rows"], got["row_number"], got["rank"], got["dense_rank"]) == 0, label
    _same(got, oracle.window_rank(keys, desc, parts))


def test_integer_narrow_and_sequence_keys(ops):
    rng = np.random.default_rng(3)
    n = 100_001
    region = rng.integers(0, 50, n).astype(np.uint32)
    status = rng.integers(-3, 4, n).astype(np.int32)
    score = rng.integers(0, 1000, n).astype(np.uint32)
    cols = [ops.Column.from_numpy(region, narrow=True), ops.Column.from_numpy(status), ops.Column.from_numpy(score),
            ops.Column.sequence(n, 5)]
    keys = [region, status, score, np.arange(5, 5 + n)]
    for parts, desc in ((1, [0, 1, 0, 0]), (2, [1, 0, 1, 1]), (0, [0, 0, 1, 0])):
        got = ops.window_rank(cols, desc, parts)
        _same(got, oracle.window_rank(keys, desc, parts))


def test_selection(ops):
    rng = np.random.default_rng(4)
    n = 300_000
    region = rng.integers(0, 20, n).astype(np.uint32)
    v = np.round(rng.lognormal(3.0, 1.0, n), 1)
    sel = np.nonzero(region % 3 == 1)[0].astype(np.uint32)
    buf = ops.DeviceBuffer(sel.nbytes, sel)
    got = ops.window_rank([ops.Column.from_numpy(region), ops.Column.from_numpy(v)], [0, 1], 1, selection=buf, count=len(sel))
    rows, rn, rk, dr = oracle.window_rank([region[sel], v[sel]], [0, 1], 1)
    assert np.array_equal(got["rows"], sel[rows])
    assert np.array_equal(got["row_number"], rn) and np.array_equal(got["rank"], rk) and np.array_equal(got["dense_rank"], dr)


def test_one_row_and_none(ops):
    one = ops.window_rank([ops.Column.from_numpy(np.array([4.5]))], [0], 0)
    assert list(one["rows"]) == [0] and list(one["row_number"]) == [1] and list(one["rank"]) == [1] and list(one["dense_rank"]) == [1]
    empty = np.zeros(0, dtype=np.uint32)
    sel = ops.DeviceBuffer(16, np.zeros(4, dtype=np.uint32))
    got = ops.window_rank([ops.Column.from_numpy(np.arange(10, dtype=np.uint32))], [0], 0, selection=sel, count=0)
    assert len(got["rows"]) == 0 and len(empty) == 0
