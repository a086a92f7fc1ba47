"""The ORDER BY oracle pinned to the reference's own sort check and tie rule (CPU only).

bench_query_sort.c holds no stored vectors: its check (pq_sort_verify, :144-178) is that the output
is a permutation of the table with the keys in order, on the table pq_load_table (:66-113) fills. The
oracle must pass that check on that table for every ORDER BY of the test (:256-268), and break ties by
input position (query_exec.c:4890-4903) with keys compared as F64 (:4859-4882).
"""
import numpy as np
import pytest

import oracle
from tests.sort_table import SORT_CASES, _mix, pq_table, verify_order


def test_generator_is_splitmix64():
    # splitmix64 from state 0: the first output mixes 0x9E3779B97F4A7C15 (public reference value)
    assert int(_mix(np.array([0x9E3779B97F4A7C15], dtype=np.uint64))[0]) == 0xE220A8397B1DCDAF


@pytest.mark.parametrize("narrow", [False, True])
@pytest.mark.parametrize("case", range(len(SORT_CASES)))
def test_oracle_passes_reference_check(case, narrow):
    t = pq_table(60000, narrow)
    keys = SORT_CASES[case]
    order = oracle.sort_rows([t[c] for c, _ in keys], [d for _, d in keys])
    assert verify_order(t, keys, order) == 0


def test_verify_catches_bad_orders():
    t = pq_table(5000, True)
    keys = [("b", 0), ("a", 1)]
    order = oracle.sort_rows([t["b"], t["a"]], [0, 1]).astype(np.int64)
    assert verify_order(t, keys, order) == 0
    swapped = order.copy()
    swapped[[10, 11]] = swapped[[11, 10]]
    assert verify_order(t, keys, swapped) != 0
    dup = order.copy()
    dup[5] = dup[6]
    assert verify_order(t, keys, dup) == 1


def test_oracle_matches_stable_lexsort():
    rng = np.random.default_rng(11)
    k1 = rng.integers(0, 20, 50000).astype(np.uint32)
    k2 = rng.integers(-5, 5, 50000).astype(np.int32)
    order = oracle.sort_rows([k1, k2], [0, 1])
    want = np.lexsort((np.arange(50000), -k2.astype(np.int64), k1))
    assert np.array_equal(order, want)


def test_ties_follow_f64_comparison():
    # -0.0 equals +0.0, and 64-bit integers that round to the same F64 tie (then go by position)
    z = np.array([0.0, -0.0, 0.0, -1.0, -0.0])
    assert list(oracle.sort_rows([z])) == [3, 0, 1, 2, 4]
    big = np.array([2**53 + 1, 2**53, 5, 2**53 + 2], dtype=np.int64)
    assert list(oracle.sort_rows([big])) == [2, 0, 1, 3]
    assert list(oracle.sort_rows([big], [1])) == [3, 0, 1, 2]
