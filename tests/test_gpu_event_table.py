"""The wide-table configuration's nine queries (10M-row, 30-column event table) against the oracle.

The table is the seeded event table at the configured 10M rows (about 1.9 GB on the device and again on the
host for the checks). Counts, integer aggregates, group keys, MIN/MAX, filter rows and the sort order
are compared exactly; f64 sums and averages within 1e-12 relative of a compensated host sum.
"""
import numpy as np
import pytest

import oracle
from tests.where_shapes import oracle_mask

pytestmark = pytest.mark.gpu

ROWS = 10_000_000


@pytest.fixture(scope="module")
def suite():
    from computeql_gb300 import build, eventbench, native, workloads
    build.build()
    native.init()
    cols, users, h, words = workloads.event_table(ROWS)
    results = {name: fn() for name, fn in eventbench.queries(cols, users, words)}
    return cols, users, h, words, results, eventbench.programs(cols, words)


def test_generator_matches_the_oracle_stream(suite):
    _, users, h, _, _, _ = suite
    from computeql_gb300 import workloads
    per_row = workloads.EVENT_DRAWS
    np.testing.assert_array_equal(h["u0"][:100_000], oracle.splitmix_u32(100_000, workloads.EVENT_SEED, per_row, 0, 1 << 20))
    np.testing.assert_array_equal(h["region"][:100_000], oracle.splitmix_u32(100_000, workloads.EVENT_SEED, per_row, 32, 50))
    np.testing.assert_array_equal(users["segment"], oracle.splitmix_u32(1_000_000, workloads.USERS_SEED, 1, 0, 20))


def test_group_by_dict_string(suite):
    _, _, h, _, res, _ = suite
    min_key, counts, sums, _, _ = res["group_by_dict_string"]
    assert min_key == 0
    np.testing.assert_array_equal(counts, np.bincount(h["s0"], minlength=200))
    np.testing.assert_array_equal(sums[:, 1], np.bincount(h["s0"], weights=h["u0"].astype(np.float64), minlength=200).astype(np.int64))


def _close(got, exact):
    return abs(got - exact) <= 1e-12 * abs(exact)


def test_group_by_status_f64(suite):
    _, _, h, _, res, _ = suite
    r = res["group_by_status_f64"]
    assert r["groups"] == 5
    for g in range(5):
        status = h["status"][int(r["repr_row"][g])]
        sel = h["status"] == status
        assert r["repr_row"][g] == np.argmax(sel)
        assert r["counts"][g] == sel.sum()
        total, m1 = oracle.compensated_sum(h["m0"][sel]), h["m1"][sel]
        assert _close(r["results"][g, 0], total)
        assert _close(r["results"][g, 1], oracle.compensated_sum(m1) / sel.sum())
        assert (r["results"][g, 2], r["results"][g, 3]) == (m1.min(), m1.max())


def test_dict_string_eq_count(suite):
    _, _, h, _, res, progs = suite
    count, rows, _ = res["dict_string_eq_filter"]
    assert rows is None
    assert count == oracle_mask(progs["eq"], dict(h)).sum() > 0


def test_group_by_region_five_aggregates(suite):
    _, _, h, _, res, _ = suite
    r = res["group_by_region_5_aggs"]
    key = h["region"]
    assert r["groups"] == 50
    for g in range(50):
        sel = key == g
        assert key[int(r["repr_row"][g])] == g and r["counts"][g] == sel.sum()
        assert r["results"][g, 0] == sel.sum()
        assert r["results"][g, 1] == float(h["u0"][sel].astype(np.int64).sum())
        assert _close(r["results"][g, 2], oracle.compensated_sum(h["m0"][sel]) / sel.sum())
        assert (r["results"][g, 3], r["results"][g, 4]) == (h["m1"][sel].min(), h["m1"][sel].max())


def test_three_predicate_count_and_sum(suite):
    _, _, h, _, res, progs = suite
    count, sums, _, _ = res["three_predicate_filter"]
    mask = oracle_mask(progs["triple"], dict(h)).astype(bool)
    assert count == mask.sum() > 0
    assert sums[0] == float(h["u5"][mask].astype(np.int64).sum())


def test_join_users_group_by_segment(suite):
    _, users, h, _, res, _ = suite
    r = res["join_users_by_segment"]
    counts, sums = oracle.join_aggregate(h["user_id"], h["u5"], users["user_id"], users["segment"], 20)
    got = {int(users["segment"][int(r["dim_row"][g])]): tuple(r["results"][g]) for g in range(r["groups"])}
    assert sorted(got) == [s for s in range(20) if counts[s]]
    for s, (count, total) in got.items():
        assert (count, total) == (float(counts[s]), float(sums[s]))


def test_group_by_user_id(suite):
    _, _, h, _, res, _ = suite
    r = res["group_by_user_id"]
    uid = h["user_id"]
    assert r["groups"] == len(np.unique(uid))
    keys = uid[r["repr_row"].astype(np.int64)]
    assert len(np.unique(keys)) == r["groups"]
    np.testing.assert_array_equal(r["counts"], np.bincount(uid, minlength=1_000_000)[keys])
    sums = np.bincount(uid, weights=h["u0"].astype(np.float64), minlength=1_000_000)
    np.testing.assert_array_equal(r["results"][:, 1], sums[keys])


def test_distinct_sessions(suite):
    _, _, h, _, res, _ = suite
    r = res["distinct_sessions"]
    assert r["groups"] == len(np.unique(h["session"]))
    assert int(r["counts"].sum()) == len(h["session"])


def test_sort_200k(suite):
    _, _, h, _, res, _ = suite
    from computeql_gb300 import eventbench
    order = res["sort_200k"]
    want_rows = np.nonzero(h["region"] == eventbench.SORT_REGION)[0]
    assert len(order) == len(want_rows)
    perm = oracle.sort_rows([h["m4"][want_rows]])
    np.testing.assert_array_equal(order, want_rows[perm.astype(np.int64)])


def test_wide_projection(suite):
    _, _, h, _, res, _ = suite
    from computeql_gb300 import eventbench
    rows, values = res["wide_projection_1pct"]
    want = np.nonzero(h["u1"] > eventbench.WIDE_U1_GT)[0]
    np.testing.assert_array_equal(rows, want)
    for name, got in zip(eventbench.STORED, values):
        np.testing.assert_array_equal(got, oracle.gather_column(h[name], want), err_msg=name)


def test_window_top3_per_region(suite):
    _, _, h, _, res, _ = suite
    from computeql_gb300 import eventbench
    sel = np.nonzero(h["u0"] > eventbench.WINDOW_U0_GT)[0]
    _, rn, _, _ = oracle.window_rank([h["region"][sel], h["u2"][sel]], desc=[0, 1], partitions=1)
    assert res["window_top3_per_region"] == int((rn <= 3).sum()) == 3 * len(np.unique(h["region"][sel]))


def test_having_over_1m_groups(suite):
    _, _, h, _, res, _ = suite
    from computeql_gb300 import eventbench
    r, keep = res["having_1m_groups"]
    keys = h["user_id"][r["repr_row"].astype(np.int64)]
    sums = np.bincount(h["user_id"], weights=h["u0"].astype(np.float64), minlength=1_000_000)
    np.testing.assert_array_equal(keep, (sums[keys] > eventbench.HAVING_SUM_GT).astype(np.uint32))


def test_eight_measures_by_region(suite):
    _, _, h, _, res, _ = suite
    from computeql_gb300 import workloads
    r = res["eight_measures_by_region"]
    assert r["groups"] == 50 and r["path"] == 3
    for g in range(50):
        sel = h["region"] == g
        for e, m in enumerate(workloads.EVENT_F64):
            assert _close(r["results"][g, e], oracle.compensated_sum(h[m][sel]))
