"""The 1B-row query suite at the size it is timed at, checked two ways (GB300 only).

1. The reference's own closed-form scale table (src/tests/scale/bench_select_scale.c:38-56: id = r + 1,
   region = r % 50, amount = r % 10000, needle_key = r * 2654435761 mod 2^32, filled on the device)
   against the reference's known answers (:97-167, restated in tests/closed_form.py) for every case of
   its case list (:1085-1170): the key lookup, the present and absent key counts, SUM/MIN/MAX, the
   0.1 % and 2 % filters, the id range, GROUP BY region, GROUP BY amount, the filtered join to the
   50-row table, the join to the 10k-row table grouped by category and the join to the 1M-row table.
2. The seed-0 table of the 1B-row configuration (splitmix64, drawn on the device) against the oracle,
   a multi-threaded C restatement of the reference's CPU operators over the same table drawn on the
   host: the seven queries bench.py times, integers bit for bit.

Each table is 3 x 4 GB on the device; the oracle's copy of the seed-0 table is 12 GB of host memory.
"""
import numpy as np
import pytest

import oracle
from tests import closed_form as cf

pytestmark = pytest.mark.gpu
N = 1_000_000_000
COUNT, SUM = 0, 1
CMP_EQ, CMP_LT, CMP_LE, CMP_GT, CMP_GE = 0, 1, 2, 3, 4          # CQLOPS_CMP_* (include/cqlops.h)


@pytest.fixture(scope="module")
def ops(gpu):
    from computeql_gb300 import ops as o
    return o


@pytest.fixture(scope="module")
def closed(ops):
    t = {"id": ops.Column.sequence(N, 1), "region": ops.Column.affine(N, 1, 0, cf.REGIONS),
         "amount": ops.Column.affine(N, 1, 0, cf.AMOUNT_RANGE), "needle": ops.Column.affine(N, cf.KEY_MULTIPLIER, 0, 0)}
    yield t
    for c in t.values():
        if c.buffer is not None:
            c.buffer.close()


def test_closed_form_columns_are_the_reference_formulas(ops, closed):
    """Spot rows of the device fills against bench_select_scale.c's loader (:176-198)."""
    rows = np.array([0, 1, 49, 50, 9999, 10000, 123_456_789, N - 1], dtype=np.int64)
    for name, want in (("region", rows % 50), ("amount", rows % 10000), ("needle", (rows * cf.KEY_MULTIPLIER) & 0xFFFFFFFF)):
        got = ops.gather_rows([closed[name]], rows=rows.astype(np.uint32))[0]
        assert np.array_equal(np.asarray(got, dtype=np.int64), want), name


def test_closed_form_key_lookups(ops, closed):
    needle_row = cf.needle_row(N)
    key = cf.key_of_row(needle_row)
    cnt, rows = ops.scan_simple([closed["needle"]], [(0, CMP_EQ, key)], want_rows=True, max_rows=16)
    assert cnt == 1 and list(rows) == [needle_row]
    absent = N + 12345
    while not cf.key_is_searchable(cf.key_of_row(absent)):
        absent += 1
    assert ops.scan_simple([closed["needle"]], [(0, CMP_EQ, cf.key_of_row(absent))])[0] == 0


def test_closed_form_scalar_cases(ops, closed):
    e = cf.expected(N)
    s, mn, mx = ops.aggregate_global([closed["amount"]])
    assert [s[0], mn[0], mx[0]] == e["sum_min_max_amount"]
    assert ops.scan_simple([closed["amount"]], [(0, CMP_GT, cf.HIGH_AMOUNT)])[0] == e["count_amount_gt_9990"]
    assert ops.scan_simple([closed["region"]], [(0, CMP_EQ, 7)])[0] == e["count_region_eq_7"]
    assert ops.scan_simple([closed["id"]], [(0, CMP_GT, 1000), (0, CMP_LE, 900_000_000)])[0] == e["count_id_range"]


def test_closed_form_group_by_region_and_amount(ops, closed):
    mk, counts, sums, _, _ = ops.group_dense(closed["region"], [COUNT, SUM], [None, closed["amount"]])
    want = np.array(cf.expected(N)["group_region"], dtype=np.float64)
    assert mk == 0 and len(counts) == 50
    assert np.array_equal(counts.astype(np.float64), want[:, 1])
    assert np.array_equal(sums[:, 1].astype(np.float64), want[:, 2])
    mk, counts, sums, _, _ = ops.group_dense(closed["amount"], [COUNT, SUM], [None, closed["region"]])
    a = np.arange(cf.AMOUNT_RANGE)
    rows = np.array([cf.amount_rows(N, int(x)) for x in a], dtype=np.int64)
    assert mk == 0 and np.array_equal(counts.astype(np.int64), rows)
    assert np.array_equal(sums[:, 1], rows * (a % cf.REGIONS))


def test_closed_form_joins(ops, closed):
    # the 50-row table filtered on its zone (regions.zone = region_id / 10 = 2)
    regions_k = np.arange(50, dtype=np.uint32)
    res = ops.join_aggregate(closed["region"], [COUNT, SUM], [None, closed["amount"]], regions_k,
                             dim_rows=np.nonzero(regions_k // 10 == 2)[0])
    assert res["groups"] == 1
    assert [res["results"][0, 0], res["results"][0, 1]] == [float(x) for x in cf.join_zone_expected(N)]
    # the 10k-row table, GROUP BY products.category (category = product_id % 20)
    products_k = np.arange(cf.AMOUNT_RANGE, dtype=np.uint32)
    category = (products_k % 20).astype(np.float64)
    res = ops.join_aggregate(closed["amount"], [COUNT], [None], products_k, group_values=[category])
    assert res["groups"] == 20
    for g in range(20):
        c = int(category[int(res["dim_row"][g])])
        assert res["results"][g, 0] == sum(cf.amount_rows(N, a) for a in range(c, cf.AMOUNT_RANGE, 20))
    # the 1M-row table: big_dim row j holds the needle_key of fact row j * (rows / 1M), weight j % 100
    j = np.arange(1_000_000, dtype=np.uint64)
    big_key = ((j * np.uint64(N // 1_000_000)) * np.uint64(cf.KEY_MULTIPLIER) & np.uint64(0xFFFFFFFF)).astype(np.uint32)
    res = ops.join_aggregate(closed["needle"], [COUNT, SUM], [None, None], big_key, dim_args=[None, (j % 100).astype(np.float64)])
    assert [res["results"][0, 0], res["results"][0, 1]] == [1_000_000.0, cf.weight_sum(1_000_000)]


@pytest.fixture(scope="module")
def seed0(ops, closed):
    from computeql_gb300 import workloads
    # the closed-form table goes first: one 1B-row table on the device at a time keeps the test within 13 GB
    for c in closed.values():
        if c.buffer is not None:
            c.buffer.close()
    t = workloads.fact_table(N)
    h = workloads.fact_numpy(N, gen=oracle.splitmix_u32)
    yield t, h
    for c in (t.region, t.amount, t.flag):
        c.buffer.close()


def test_seed0_suite_matches_the_oracle(ops, seed0):
    """bench.py's seven queries over the seed-0 1B-row table, each against the oracle."""
    import bench
    from computeql_gb300 import workloads
    t, h = seed0
    d50, d1m = workloads.dim_tables()
    key = 987_654_321
    got = {name: q() for name, _, q in bench.make_queries(ops, t, key, (d50, d1m))}

    s, mn, mx = got["sum_min_max_amount"]
    assert (s[0], mn[0], mx[0]) == oracle.aggregate_global_cpu(h["amount"])
    assert got["count_flag_lt_2"][0] == oracle.scan_and([(h["flag"], CMP_LT, 2)], N)[0]

    mk, counts, sums, _, _ = got["group_by_region"]
    ec, es, _, _ = oracle.group_dense(h["region"], mk, len(counts), [SUM, COUNT], [h["amount"], None])
    assert np.array_equal(counts, ec) and np.array_equal(sums[:, 0], es[:, 0])
    mk, counts, sums, _, _ = got["group_by_amount_10k"]
    ec, es, _, _ = oracle.group_dense(h["amount"], mk, len(counts), [COUNT, SUM], [None, h["region"]])
    assert np.array_equal(counts, ec) and np.array_equal(sums[:, 1], es[:, 1])

    cnt, rows = got["point_lookup_id"]
    assert cnt == 1 and list(rows) == [key]

    keep = np.where(d50["name_id"] == 3, 0, 0xFFFFFFFF).astype(np.uint32)
    ec, es = oracle.join_aggregate(h["region"], h["amount"], d50["k"], keep, 1)
    r = got["join_dim50_filtered"]
    assert r["groups"] == 1 and [r["results"][0, 0], r["results"][0, 1]] == [float(ec[0]), float(es[0])]

    ec, es = oracle.join_aggregate(h["amount"], h["amount"], d1m["k"], d1m["seg"], 20)
    r = got["join_dim1m_group_by_seg"]
    assert r["groups"] == 20
    for g in range(20):
        seg = int(d1m["seg"][int(r["dim_row"][g])])
        assert [r["results"][g, 0], r["results"][g, 1]] == [float(es[seg]), float(ec[seg])]
