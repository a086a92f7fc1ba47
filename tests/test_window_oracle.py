"""The window-rank oracle against the reference's own check (bench_query_window_rank.c:40-104) on its
test table and all nine of its cases (CPU only)."""
import numpy as np
import pytest

import oracle
from tests.window_table import CASES, tables, verify


@pytest.mark.parametrize("case", CASES, ids=[c[0] for c in CASES])
def test_oracle_passes_the_reference_check(case):
    label, nk, parts, mask, narrow = case
    wide, nar = tables(20000)
    keys = (nar if narrow else wide)[:nk]
    desc = [(mask >> k) & 1 for k in range(nk)]
    rows, rn, rk, dr = oracle.window_rank(keys, desc, parts)
    assert verify(keys, desc, parts, rows, rn, rk, dr) == 0, label


def test_ties_and_partitions_by_hand():
    part = np.array([1, 0, 1, 0, 1, 0], dtype=np.float64)
    order = np.array([5, 7, 5, 7, 3, 7], dtype=np.float64)
    rows, rn, rk, dr = oracle.window_rank([part, order], [0, 0], 1)
    # partition 0: rows 1, 3, 5 all order 7 -> peers; partition 1: rows 4 (3), 0 and 2 (5)
    assert list(rows) == [1, 3, 5, 4, 0, 2]
    assert list(rn) == [1, 2, 3, 1, 2, 3]
    assert list(rk) == [1, 1, 1, 1, 2, 2]
    assert list(dr) == [1, 1, 1, 1, 2, 2]
