"""The fixed-point oracle pinned on the reference's own GROUP BY table (CPU only).

bench_query_agg_resident.c builds t (:50-60, :293-298: 500k rows from the bench generator seeded
0xA66E5EED, three draws per row: grp = draw % 40, wv = draw % 1001, dv = (draw % 10000) / 100.0) and
checks "SELECT grp, SUM(dv), MIN(dv), MAX(dv) FROM t GROUP BY grp" (:205) against SQLite. dv has two
places, so the reference takes the fixed-point path: its answers are the exact cent totals divided
by 100. The oracle must give exactly those, find scale 2, and refuse a column that is no decimal.
"""
import numpy as np

import oracle
from tests.bench_rng import rows

AR_ROWS, AR_GROUPS = 500000, 40


def ar_table():
    r = rows(0xA66E5EED, AR_ROWS, 3)
    grp = (r[:, 0] % np.uint64(AR_GROUPS)).astype(np.uint32)
    wv = (r[:, 1] % np.uint64(1001)).astype(np.float64)
    cents = (r[:, 2] % np.uint64(10000)).astype(np.int64)
    return grp, wv, cents, cents / 100.0


def test_scale_of_the_decimal_column():
    _, wv, _, dv = ar_table()
    assert oracle.fixed_scale(dv)[0] == 2
    assert oracle.fixed_scale(wv)[0] == 0


def test_group_by_decimal_is_exact():
    grp, _, cents, dv = ar_table()
    got = oracle.dense_fixed(grp.astype(np.float64), [1, 3, 4], [dv, dv, dv], [2, 2, 2])
    assert list(got["keys"]) == list(range(AR_GROUPS))
    for g in range(AR_GROUPS):
        m = grp == g
        assert got["counts"][g] == m.sum()
        assert got["first_rows"][g] == np.nonzero(m)[0][0]
        assert got["results"][g, 0] == float(cents[m].sum()) / 100.0
        assert got["results"][g, 1] == float(cents[m].min()) / 100.0
        assert got["results"][g, 2] == float(cents[m].max()) / 100.0
        # and within rounding of a plain f64 sum in row order (what SQLite computes)
        assert abs(got["results"][g, 0] - np.add.reduce(dv[m])) <= 1e-9 * abs(got["results"][g, 0])


def test_scale_edge_cases():
    assert oracle.fixed_scale([])[0] == 0
    assert oracle.fixed_scale([0.1, 0.25, 0.125])[0] == 3
    assert oracle.fixed_scale([1e-6])[0] == 6
    assert oracle.fixed_scale([1e-7])[0] == -1
    assert oracle.fixed_scale([2147.483647])[0] == 6
    assert oracle.fixed_scale([2147.483648])[0] == -1          # 2147483648 is not below 2^31
    assert oracle.fixed_scale([2.0**31])[0] == -1
    assert oracle.fixed_scale([np.nan])[0] == -1
    assert list(oracle.fixed_scale_each([0.5, 1.0 / 3.0, -2.75, np.inf])) == [1, -1, 2, -1]
