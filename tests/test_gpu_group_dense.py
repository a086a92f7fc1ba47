"""aggregate_dense_native through the C ABI against the oracle and the closed forms (bit-exact)."""
import json
import os

import numpy as np
import pytest

import oracle
from tests import closed_form as cf

pytestmark = pytest.mark.gpu
GOLDEN = os.path.join(os.path.dirname(__file__), "golden")
COUNT, SUM, AVG, MIN, MAX = 0, 1, 2, 3, 4


@pytest.fixture(scope="module")
def ops(gpu):
    from computeql_gb300 import ops as o
    return o


def test_c1_group_by_region_matches_golden(ops):
    from computeql_gb300 import workloads
    fx = json.load(open(os.path.join(GOLDEN, "c1_oracle.json")))
    t = workloads.fact_table(fx["rows"])
    mk, counts, sums, _, _ = ops.group_dense(t.region, [SUM, COUNT], [t.amount, None])
    got = [[mk + g, int(sums[g, 0]), int(counts[g])] for g in range(len(counts))]
    assert got == fx["group_region_sum_amount_count"]


@pytest.mark.parametrize("n", [1, 49, 50, 51, 10001, 1000003, 4_000_000])
def test_closed_form_group_by_region_and_amount(ops, n):
    _, region, amount, _ = oracle.closed_form(n)
    exp = cf.expected(n)
    r = ops.Column.from_numpy(region)
    a = ops.Column.from_numpy(amount)
    mk, counts, sums, _, _ = ops.group_dense(r, [COUNT, SUM], [None, a])
    got = [[mk + g, int(counts[g]), float(sums[g, 1])] for g in range(len(counts)) if counts[g]]
    assert got == exp["group_region"]
    mk, counts, sums, _, _ = ops.group_dense(a, [COUNT, SUM], [None, r])
    got = [[mk + g, int(counts[g]), int(sums[g, 1])] for g in range(len(counts)) if counts[g]]
    assert got == exp["group_amount"]


def _check(ops, key, funcs, args, narrow=False):
    kcol = ops.Column.from_numpy(key, narrow=narrow)
    uploaded = {}
    for a in args:
        if a is not None and id(a) not in uploaded:
            uploaded[id(a)] = ops.Column.from_numpy(a, narrow=narrow)
    dargs = [uploaded[id(a)] if a is not None else None for a in args]
    mk, counts, sums, mins, maxs = ops.group_dense(kcol, funcs, dargs)
    groups = len(counts)
    ec, es, emin, emax = oracle.group_dense(key, mk, groups, funcs, args)
    assert np.array_equal(counts, ec)
    for e, f in enumerate(funcs):
        if f in (SUM, AVG):
            assert np.array_equal(sums[:, e], es[:, e])
        if f == MIN:
            assert np.array_equal(mins[:, e], emin[:, e])
        if f == MAX:
            assert np.array_equal(maxs[:, e], emax[:, e])


@pytest.mark.parametrize("groups", [1, 5, 50, 200, 1000, 10000, 65536])
def test_group_counts_and_all_functions(ops, groups):
    n = 700_001
    rng = np.random.default_rng(groups)
    key = rng.integers(0, groups, n).astype(np.uint32)
    v = rng.integers(0, 1 << 31, n).astype(np.uint32)
    w = rng.integers(-2**31, 2**31, n).astype(np.int32)
    if groups <= 1000:
        _check(ops, key, [COUNT, SUM, MIN, MAX, SUM, AVG, MIN, MAX], [None, v, v, v, w, w, w, w])
    else:
        # the reference caps a dense group-by at 256 tiles of its 2048-word slices (query_exec.c:7739-7743)
        _check(ops, key, [COUNT, SUM], [None, v])
        if groups <= 10000:
            _check(ops, key, [MIN, MAX], [w, w])


def test_refuses_what_the_reference_refuses(ops):
    n = 1000
    key = (np.arange(n) % 65536).astype(np.uint32)
    key[-1] = 65535
    w = np.arange(n, dtype=np.int32)
    with pytest.raises(ops.OpError, match="256 tiles"):
        _check(ops, key, [MIN, MAX], [w, w])


def test_signed_keys_with_negative_minimum(ops):
    n = 300_007
    rng = np.random.default_rng(9)
    key = rng.integers(-1000, 1000, n).astype(np.int32)
    v = rng.integers(-100, 100, n).astype(np.int32)
    _check(ops, key, [SUM, COUNT, MAX], [v, None, v])


@pytest.mark.parametrize("n", [1, 3, 4, 5, 17, 1023])
def test_ragged_row_counts(ops, n):
    rng = np.random.default_rng(n)
    key = rng.integers(10, 20, n).astype(np.uint32)
    v = rng.integers(0, 10, n).astype(np.uint32)
    _check(ops, key, [COUNT, SUM, MIN], [None, v, v])


def test_narrow_key_and_arguments(ops):
    n = 1_000_003
    rng = np.random.default_rng(21)
    key = (1000 + rng.integers(0, 200, n)).astype(np.uint32)
    v = (50000 + rng.integers(0, 60000, n)).astype(np.uint32)
    w = (-7 + rng.integers(0, 100, n)).astype(np.int32)
    _check(ops, key, [COUNT, SUM, MIN, MAX, SUM], [None, v, v, v, w], narrow=True)


def test_sequence_argument(ops):
    n = 100_000
    key = (np.arange(n) % 7).astype(np.uint32)
    kcol = ops.Column.from_numpy(key)
    seq = ops.Column.sequence(n, 10)
    mk, counts, sums, _, _ = ops.group_dense(kcol, [SUM], [seq])
    ids = np.arange(n, dtype=np.int64) + 10
    exp = [int(ids[key == g].sum()) for g in range(7)]
    assert [int(x) for x in sums[:, 0]] == exp


def test_large_sums_wrap_like_two_words(ops):
    # sums past 2^32 need the high word; every row near 2^32 - 1
    n = 2_000_000
    key = np.zeros(n, dtype=np.uint32)
    v = np.full(n, 0xFFFFFFF0, dtype=np.uint32)
    _check(ops, key, [SUM], [v])


@pytest.mark.parametrize("dtype,lo,hi", [(np.uint32, 0, 10000), (np.int32, -3000, 3000), (np.uint32, 2**31 - 600, 2**31 - 1)])
def test_key_as_its_own_argument(ops, dtype, lo, hi):
    # GROUP BY amount ... SUM(amount): the argument column is the key column (read once, SUM = key x count)
    rng = np.random.default_rng(17)
    key = rng.integers(lo, hi, 2_000_003).astype(dtype)
    funcs = [SUM, COUNT, MIN, MAX, AVG]
    _check(ops, key, funcs, [key if f != COUNT else None for f in funcs])


@pytest.mark.parametrize("arg_range", [(0, 50), (-1000, 1000), (0, 100_000), (0, 2**31 - 1)])
@pytest.mark.parametrize("groups", [7, 10000])
def test_count_and_sum_of_one_argument(ops, arg_range, groups):
    # COUNT/SUM/AVG of one column: packed into one shared word per group when a CTA cannot carry past 2^31
    rng = np.random.default_rng(groups + arg_range[1])
    n = 20_000_003
    key = rng.integers(0, groups, n).astype(np.uint32)
    arg = rng.integers(arg_range[0], arg_range[1], n)
    arg = arg.astype(np.int32 if arg_range[0] < 0 else np.uint32)
    _check(ops, key, [COUNT, SUM, AVG, SUM], [None, arg, arg, arg])
