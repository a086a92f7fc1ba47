"""The wide-table configuration's nine queries (10M-row, 30-column event table) against the oracle.

The table is the seeded event table at 1M rows (the generator is the same at 10M; the 1M-group query keeps
its 1M possible user ids). Counts, integer aggregates, group keys, filter rows and the sort order are
compared exactly; f64 sums within 1e-12 relative of a compensated host sum; the distinct count equals the
oracle's HyperLogLog estimate from its own registers.
"""
import numpy as np
import pytest

import oracle
from tests.where_shapes import oracle_mask

pytestmark = pytest.mark.gpu

ROWS = 1_000_000


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
    min_key, counts, _, _, _ = res["group_by_dict_string"]
    assert min_key == 0
    np.testing.assert_array_equal(counts, np.bincount(h["s0"], minlength=200))


def test_group_by_status_f64_sums(suite):
    _, _, h, _, res, _ = suite
    r = res["group_by_status_f64"]
    assert r["groups"] == 5
    for g in range(5):
        status = h["status"][int(r["repr_row"][g])]
        sel = h["status"] == status
        assert r["counts"][g] == sel.sum()
        for e, m in enumerate(("m0", "m1", "m2")):
            exact = oracle.compensated_sum(h[m][sel])
            assert abs(r["results"][g, e] - exact) <= 1e-12 * abs(exact)


@pytest.mark.parametrize("name,program", [("dict_string_eq_filter", "eq"), ("three_predicate_filter", "triple")])
def test_filters(suite, name, program):
    cols, _, h, _, res, progs = suite
    count, rows, _ = res[name]
    arrays = {k: v for k, v in h.items()}
    want = np.nonzero(oracle_mask(progs[program], arrays))[0]
    assert count == len(want) and len(want) > 0
    np.testing.assert_array_equal(rows, want)


def test_group_by_region_five_aggregates(suite):
    _, _, h, _, res, _ = suite
    min_key, counts, sums, mins, maxs = res["group_by_region_5_aggs"]
    assert min_key == 0 and len(counts) == 50
    key = h["region"]
    np.testing.assert_array_equal(counts, np.bincount(key, minlength=50))
    for g in range(50):
        sel = key == g
        assert sums[g, 1] == h["u0"][sel].astype(np.int64).sum()
        assert mins[g, 2] == h["u1"][sel].min()
        assert maxs[g, 3] == h["u2"][sel].max()
        assert sums[g, 4] == h["u3"][sel].astype(np.int64).sum()      # AVG's sum; the average is sum / count


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
    present = np.unique(uid)
    assert r["groups"] == len(present)
    keys = uid[r["repr_row"].astype(np.int64)]
    assert len(np.unique(keys)) == r["groups"]
    order = np.argsort(uid, kind="stable")
    starts = np.searchsorted(uid[order], keys)
    ends = np.searchsorted(uid[order], keys, side="right")
    np.testing.assert_array_equal(r["counts"], ends - starts)
    m0 = h["m0"][order]
    for g in np.random.default_rng(1).choice(r["groups"], 2000, replace=False):
        exact = oracle.compensated_sum(m0[starts[g]:ends[g]])
        assert abs(r["results"][g, 1] - exact) <= 1e-12 * abs(exact)


def test_approx_distinct_session(suite):
    _, _, h, _, res, _ = suite
    r = res["approx_distinct_session"]
    want = round(oracle.hll_estimate(oracle.hll_registers(h["session"].astype(np.float64))))
    assert r["results"][0, 0] == want


def test_order_by_f64_filtered(suite):
    _, _, h, _, res, _ = suite
    rows, order = res["order_by_f64_filtered"]
    want_rows = np.nonzero((h["region"] < 5) & (h["status"] == 1))[0]
    np.testing.assert_array_equal(rows, want_rows)
    perm = oracle.sort_rows([h["m4"][want_rows]])
    np.testing.assert_array_equal(order, want_rows[perm.astype(np.int64)])
