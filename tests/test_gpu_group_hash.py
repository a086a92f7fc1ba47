"""Hash GROUP BY, HyperLogLog and t-digest through the C ABI against the oracle.

Counts, whole-number sums, minimums, maximums and group membership are bit-exact; f64 sums within
1e-12 relative; HyperLogLog registers equal the oracle's bit for bit (per group and global, p = 10, up to
4M distinct values), and the estimates stay within the reference's 3 x 1.04 / sqrt(2^10) bound
(src/tests/bench_query_approx_agg.c:174-179); t-digest percentiles within the reference's 5 %
(:265-270); the exact edge cases 1 row -> 1 and all-identical -> 1 (:428-478).
"""
import math

import numpy as np
import pytest

import oracle

pytestmark = pytest.mark.gpu
COUNT, SUM, AVG, MIN, MAX, ACD, PCT = 0, 1, 2, 3, 4, 5, 6
HLL_BOUND = 3 * 1.04 / math.sqrt(1024)


@pytest.fixture(scope="module")
def ops(gpu):
    from computeql_gb300 import ops as o
    return o


def by_key(res, key_arrays):
    """group results keyed by the key values of each group's representative row"""
    out = {}
    for g in range(res["groups"]):
        r = int(res["repr_row"][g])
        out[tuple(k[r].item() for k in key_arrays)] = (int(res["counts"][g]), res["results"][g])
    return out


@pytest.mark.parametrize("path", [0, 1])
@pytest.mark.parametrize("groups", [1, 7, 1000, 100_000])
def test_integer_aggregates_per_group(ops, path, groups):
    n = 1_000_003
    rng = np.random.default_rng(groups)
    key = rng.integers(0, groups, n).astype(np.uint32)
    v = rng.integers(0, 1 << 20, n).astype(np.uint32)
    w = rng.integers(-(1 << 20), 1 << 20, n).astype(np.int32)
    kc, vc, wc = ops.Column.from_numpy(key), ops.Column.from_numpy(v), ops.Column.from_numpy(w)
    res = ops.group_hash([kc], [COUNT, SUM, MIN, MAX, SUM, AVG], [None, vc, vc, vc, wc, wc], path=path)
    # path 0 picks the direct tables for a key range past 65536 values, else the fixed-point reduce
    assert res["path"] == ((4 if groups > 65536 else 2) if path == 0 else 1)
    got = by_key(res, [key])
    uniq = np.unique(key)
    assert len(got) == len(uniq)
    order = np.argsort(key, kind="stable")
    ks = key[order]
    starts = np.searchsorted(ks, uniq)
    ends = np.searchsorted(ks, uniq, side="right")
    for u, s, e in zip(uniq, starts, ends):
        rows = order[s:e]
        cnt, r = got[(int(u),)]
        assert cnt == e - s
        assert r[0] == e - s
        assert r[1] == float(v[rows].astype(np.int64).sum())
        assert (r[2], r[3]) == (float(v[rows].min()), float(v[rows].max()))
        ws = float(w[rows].astype(np.int64).sum())
        assert r[4] == ws
        assert r[5] == ws / (e - s)


def test_two_keys_and_f64_arguments(ops):
    n = 400_001
    rng = np.random.default_rng(5)
    k1 = rng.integers(0, 30, n).astype(np.uint32)
    k2 = rng.integers(-5, 5, n).astype(np.int32)
    d = rng.lognormal(3.0, 1.0, n)
    res = ops.group_hash([ops.Column.from_numpy(k1), ops.Column.from_numpy(k2)], [SUM, MIN, MAX, COUNT], [ops.Column.from_numpy(d)] * 3 + [None])
    dcol_res = by_key(res, [k1, k2])
    assert len(dcol_res) == len(set(zip(k1.tolist(), k2.tolist())))
    for (a, b), (cnt, r) in dcol_res.items():
        sel = d[(k1 == a) & (k2 == b)]
        assert cnt == len(sel) and r[3] == len(sel)
        exact = math.fsum(sel)
        assert abs(r[0] - exact) <= 1e-12 * abs(exact)
        assert (r[1], r[2]) == (sel.min(), sel.max())


def test_string_keys(ops):
    n = 200_000
    rng = np.random.default_rng(8)
    words = ["north", "south", "east", "west", "centre", "", "x" * 40]
    vals = [words[i] for i in rng.integers(0, len(words), n)]
    v = rng.integers(0, 100, n).astype(np.uint32)
    sc = ops.StringColumn(vals)
    res = ops.group_hash([sc], [COUNT, SUM], [None, ops.Column.from_numpy(v)])
    assert res["groups"] == len(set(vals))
    arr = np.array(vals, dtype=object)
    for g in range(res["groups"]):
        name = vals[int(res["repr_row"][g])]
        sel = arr == name
        assert res["counts"][g] == sel.sum()
        assert res["results"][g, 1] == float(v[sel].astype(np.int64).sum())


@pytest.mark.parametrize("distinct", [1, 2, 100, 5000, 4_000_000])
def test_hll_global_matches_oracle_registers(ops, distinct):
    n = 2_000_000 if distinct < 4_000_000 else 10_000_000
    rng = np.random.default_rng(distinct)
    session = rng.integers(0, distinct, n).astype(np.uint32)
    res = ops.group_hash([], [ACD], [ops.Column.from_numpy(session)])
    assert res["groups"] == 1
    regs = ops.group_hash_registers()
    want_regs = oracle.hll_registers(session.astype(np.float64))
    assert regs.shape == (1, 1024)
    assert np.array_equal(regs[0], want_regs)          # registers bit for bit, not just the estimate
    est = res["results"][0, 0]
    assert est == round(oracle.hll_estimate(want_regs))
    true = len(np.unique(session))
    assert abs(est - true) <= HLL_BOUND * true


def test_hll_per_group_matches_oracle(ops):
    n = 1_000_000
    rng = np.random.default_rng(77)
    key = rng.integers(0, 10, n).astype(np.uint32)
    val = rng.integers(0, 50_000, n).astype(np.uint32)
    res = ops.group_hash([ops.Column.from_numpy(key)], [ACD, COUNT], [ops.Column.from_numpy(val), None])
    regs = ops.group_hash_registers()
    assert regs.shape == (res["groups"], 1024)
    for g in range(res["groups"]):
        k = key[int(res["repr_row"][g])]
        sel = val[key == k].astype(np.float64)
        want_regs = oracle.hll_registers(sel)
        assert np.array_equal(regs[g], want_regs)
        assert res["results"][g, 0] == round(oracle.hll_estimate(want_regs))
        assert res["results"][g, 1] == len(sel)


def test_hll_two_sketches_per_group_registers(ops):
    """Two APPROX_COUNT_DISTINCT expressions over different columns: registers laid out [group][expr][1024]."""
    n = 500_000
    rng = np.random.default_rng(91)
    key = rng.integers(0, 4, n).astype(np.uint32)
    a = rng.integers(0, 300_000, n).astype(np.uint32)
    b = rng.normal(0.0, 1e6, n)
    res = ops.group_hash([ops.Column.from_numpy(key)], [ACD, COUNT, ACD],
                         [ops.Column.from_numpy(a), None, ops.Column.from_numpy(b)])
    regs = ops.group_hash_registers()
    assert regs.shape == (2 * res["groups"], 1024)
    for g in range(res["groups"]):
        sel = key == key[int(res["repr_row"][g])]
        assert np.array_equal(regs[2 * g], oracle.hll_registers(a[sel].astype(np.float64)))
        assert np.array_equal(regs[2 * g + 1], oracle.hll_registers(b[sel]))


def test_hll_exact_edge_cases(ops):
    one = ops.Column.from_numpy(np.array([42], dtype=np.uint32))
    assert ops.group_hash([], [ACD], [one])["results"][0, 0] == 1
    same = ops.Column.from_numpy(np.full(100_000, 7, dtype=np.uint32))
    assert ops.group_hash([], [ACD], [same])["results"][0, 0] == 1
    empty = ops.Column.from_numpy(np.zeros(0, dtype=np.uint32))
    assert ops.group_hash([], [ACD], [empty])["groups"] == 0


@pytest.mark.parametrize("fraction", [0.1, 0.5, 0.9, 0.99])
def test_tdigest_within_five_percent(ops, fraction):
    n = 1_000_000
    rng = np.random.default_rng(int(fraction * 100))
    d = rng.lognormal(3.0, 1.0, n)
    res = ops.group_hash([], [PCT], [ops.Column.from_numpy(d)], params=[fraction])
    exact = float(np.quantile(d, fraction))
    assert abs(res["results"][0, 0] - exact) <= 0.05 * exact


def test_tdigest_single_row_and_grouped(ops):
    one = ops.Column.from_numpy(np.array([3.25]))
    assert ops.group_hash([], [PCT], [one], params=[0.5])["results"][0, 0] == 3.25
    n = 500_000
    rng = np.random.default_rng(3)
    key = rng.integers(0, 5, n).astype(np.uint32)
    d = rng.random(n) * 100
    res = ops.group_hash([ops.Column.from_numpy(key)], [PCT, COUNT], [ops.Column.from_numpy(d), None], params=[0.5, 0.5])
    for g in range(res["groups"]):
        k = key[int(res["repr_row"][g])]
        exact = float(np.median(d[key == k]))
        assert abs(res["results"][g, 0] - exact) <= 0.05 * exact


def test_tdigest_estimator_matches_the_oracle_on_fixed_centroids():
    from computeql_gb300 import native
    import ctypes as C
    rng = np.random.default_rng(1)
    m = rng.random(1000).astype(np.float32)
    w = rng.integers(1, 20, 1000).astype(np.float32)
    for f in (0.0, 0.01, 0.5, 0.77, 1.0):
        a, b = m.copy(), w.copy()
        got = native.load_ops().cqlops_tdigest_percentile(a.ctypes.data, b.ctypes.data, len(a), f)
        assert got == oracle.tdigest_percentile(m, w, f)


def test_small_table_grows_buckets_on_overflow(ops):
    # 200k distinct keys in 400k rows: the first table (rows/64 buckets) overflows and is grown
    n = 400_000
    key = (np.arange(n) % 200_000).astype(np.uint32)
    res = ops.group_hash([ops.Column.from_numpy(key)], [COUNT], [None])
    assert res["groups"] == 200_000
    assert np.all(res["counts"] == 2)


def test_decimal_arguments_take_the_fixed_path(ops):
    # f64 decimals of at most 6 places reduce as scaled integers (aggregate_hash_reduce_fixed with the
    # found scale), finalized as the reference does: bit for bit what the fixed-point oracle gives
    n = 1_000_003
    rng = np.random.default_rng(31)
    key = rng.integers(0, 1000, n).astype(np.uint32)
    price = rng.integers(-10**7, 10**7, n) / 100.0
    qty = rng.integers(0, 10**4, n) / 1000.0
    pc, qc = ops.Column.from_numpy(price), ops.Column.from_numpy(qty)
    funcs = [COUNT, SUM, AVG, MIN, MAX, SUM]
    res = ops.group_hash([ops.Column.from_numpy(key)], funcs, [None, pc, pc, pc, pc, qc])
    assert res["path"] == 2
    want = oracle.dense_fixed(key.astype(np.float64), funcs, [None, price, price, price, price, qty], [0, 2, 2, 2, 2, 3])
    got = {int(key[int(res["repr_row"][g])]): res["results"][g] for g in range(res["groups"])}
    assert len(got) == len(want["keys"])
    for i, k in enumerate(want["keys"]):
        assert np.array_equal(got[int(k)].view(np.uint64), want["results"][i].view(np.uint64))


def test_million_groups(ops):
    # GROUP BY user_id over 10M rows (the 30-column event table's 1M-group query)
    n = 10_000_000
    rng = np.random.default_rng(41)
    user = rng.integers(0, 1_000_000, n).astype(np.uint32)
    measure = rng.lognormal(3.0, 1.0, n)
    res = ops.group_hash([ops.Column.from_numpy(user)], [COUNT, SUM], [None, ops.Column.from_numpy(measure)], group_hint=1_000_000)
    assert res["path"] == 1
    keys = user[res["repr_row"].astype(np.int64)]
    assert len(np.unique(keys)) == res["groups"] == len(np.unique(user))
    counts = np.bincount(user, minlength=1_000_000)
    sums = np.bincount(user, weights=measure, minlength=1_000_000)
    assert np.array_equal(res["results"][:, 0], counts[keys].astype(np.float64))
    assert np.array_equal(res["counts"], counts[keys].astype(np.uint64))
    assert np.all(np.abs(res["results"][:, 1] - sums[keys]) <= 1e-11 * sums[keys])
    for g in range(0, res["groups"], 99991):
        exact = math.fsum(measure[user == keys[g]])
        assert abs(res["results"][g, 1] - exact) <= 1e-12 * exact


@pytest.mark.parametrize("groups", [1, 3, 5])
def test_few_groups_many_rows(ops, groups):
    # every lane of a warp on a handful of groups: warp-aggregated counts, cursors and sums
    n = 5_000_000
    rng = np.random.default_rng(groups)
    key = rng.integers(0, groups, n).astype(np.uint32)
    v = rng.integers(-1000, 1000, n).astype(np.int32)
    d = rng.random(n)
    kc, vc, dc = ops.Column.from_numpy(key), ops.Column.from_numpy(v), ops.Column.from_numpy(d)
    fixed = ops.group_hash([kc], [COUNT, SUM, MIN, MAX], [None, vc, vc, vc])
    assert fixed["path"] == 2
    csr = ops.group_hash([kc], [COUNT, SUM], [None, dc], path=1)
    assert csr["path"] == 1
    for g in range(fixed["groups"]):
        k = key[int(fixed["repr_row"][g])]
        m = key == k
        assert list(fixed["results"][g]) == [m.sum(), float(v[m].astype(np.int64).sum()), float(v[m].min()), float(v[m].max())]
    for g in range(csr["groups"]):
        k = key[int(csr["repr_row"][g])]
        exact = math.fsum(d[key == k])
        assert abs(csr["results"][g, 1] - exact) <= 1e-12 * exact
    # automatic: a key of few values with f64 sums goes through the shared scan (path 3), groups in key
    # order, each represented by its first row
    small = ops.group_hash([kc], [COUNT, SUM, AVG], [None, dc, dc])
    assert small["path"] == 3
    present = np.unique(key)
    assert small["groups"] == len(present)
    for g, k in enumerate(present):
        m = key == k
        assert small["repr_row"][g] == np.argmax(m)
        exact = math.fsum(d[m])
        assert small["counts"][g] == m.sum() and small["results"][g, 0] == m.sum()
        assert abs(small["results"][g, 1] - exact) <= 1e-12 * exact
        assert abs(small["results"][g, 2] - exact / m.sum()) <= 1e-12 * exact / m.sum()


@pytest.mark.parametrize("span", [70_000, 1_000_000])
def test_direct_tables_for_a_dense_key_range(ops, span):
    # one i32 key over a range past the dense group-by's 65536 values, not every value present, negative keys
    # and arguments: groups in key order, each represented by its first row
    n = 2_000_003
    rng = np.random.default_rng(span)
    key = (rng.integers(0, span, n) - span // 3).astype(np.int32)
    key[:2] = [-(span // 3), span - 1 - span // 3]          # the range's ends present
    v = rng.integers(-(1 << 30), 1 << 30, n).astype(np.int32)
    u = rng.integers(0, 1 << 20, n).astype(np.uint32)
    kc, vc, uc = ops.Column.from_numpy(key), ops.Column.from_numpy(v), ops.Column.from_numpy(u)
    funcs = [COUNT, SUM, AVG, MIN, MAX, SUM]
    res = ops.group_hash([kc], funcs, [None, vc, vc, vc, vc, uc])
    assert res["path"] == 4
    uniq, first, counts = np.unique(key, return_index=True, return_counts=True)
    assert res["groups"] == len(uniq)
    np.testing.assert_array_equal(res["repr_row"], first)
    np.testing.assert_array_equal(res["counts"], counts)
    order = np.argsort(key, kind="stable")
    bounds = np.concatenate([[0], np.cumsum(counts)])
    vsum = np.add.reduceat(v[order].astype(np.int64), bounds[:-1])
    usum = np.add.reduceat(u[order].astype(np.int64), bounds[:-1])
    np.testing.assert_array_equal(res["results"][:, 0], counts.astype(np.float64))
    np.testing.assert_array_equal(res["results"][:, 1], vsum.astype(np.float64))
    np.testing.assert_array_equal(res["results"][:, 2], vsum.astype(np.float64) / counts)
    np.testing.assert_array_equal(res["results"][:, 3], np.minimum.reduceat(v[order], bounds[:-1]).astype(np.float64))
    np.testing.assert_array_equal(res["results"][:, 4], np.maximum.reduceat(v[order], bounds[:-1]).astype(np.float64))
    np.testing.assert_array_equal(res["results"][:, 5], usum.astype(np.float64))
    # too small a result area is refused, not overrun; a range this path does not take is refused when asked for
    with pytest.raises(ops.OpError):
        ops.group_hash([kc], funcs, [None, vc, vc, vc, vc, uc], max_groups=len(uniq) - 1)
    small = ops.Column.from_numpy(rng.integers(0, 1000, n).astype(np.uint32))
    with pytest.raises(ops.OpError):
        ops.group_hash([small], [COUNT], [None], path=4)


@pytest.mark.parametrize("seed", range(4))
def test_direct_tables_random_shapes(ops, seed):
    # random dense key ranges past 65536 values, sparse use of them, and random aggregate mixes
    rng = np.random.default_rng(200 + seed)
    span = int(rng.integers(65_537, 3_000_000))
    n = int(rng.integers(span // 8 + 1, 3_000_000))
    low = int(rng.integers(-2**30, 2**30))
    key = (rng.integers(0, span, n) + low).astype(np.int32)
    key[0], key[-1] = low, low + span - 1
    arrs = [rng.integers(-2**31, 2**31 - 1, n).astype(np.int32), rng.integers(0, 2**31 - 1, n).astype(np.uint32)]
    cols = [ops.Column.from_numpy(a) for a in arrs]
    funcs = [int(f) for f in rng.integers(0, 5, int(rng.integers(1, 9)))]
    which = [int(w) for w in rng.integers(0, 2, len(funcs))]
    res = ops.group_hash([ops.Column.from_numpy(key)], funcs, [None if f == COUNT else cols[w] for f, w in zip(funcs, which)])
    assert res["path"] == 4
    uniq, first, counts = np.unique(key, return_index=True, return_counts=True)
    np.testing.assert_array_equal(res["repr_row"], first)
    np.testing.assert_array_equal(res["counts"], counts)
    order = np.argsort(key, kind="stable")
    starts = np.concatenate([[0], np.cumsum(counts)])[:-1]
    for e, (f, w) in enumerate(zip(funcs, which)):
        got = res["results"][:, e]
        if f == COUNT:
            np.testing.assert_array_equal(got, counts.astype(np.float64))
            continue
        v = arrs[w][order]
        if f in (SUM, AVG):
            s = np.add.reduceat(v.astype(np.int64), starts).astype(np.float64)
            np.testing.assert_array_equal(got, s if f == SUM else s / counts)
        else:
            m = (np.minimum if f == MIN else np.maximum).reduceat(v, starts)
            np.testing.assert_array_equal(got, m.astype(np.float64))
