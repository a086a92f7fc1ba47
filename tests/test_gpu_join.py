"""Hash joins and the join-aggregate pushdown through the C ABI.

Join output is compared as sorted (probe, build) pairs with a join computed independently on the
host; the pushdown against the reference's own closed-form answers (the joins of
src/tests/scale/bench_select_scale.c:1158-1170: the 50-row table filtered on its zone, the 1M-row
table on the needle key) and against numpy on the 1B-row configuration's tables at 10M rows.
"""
import numpy as np
import pytest

import oracle
from tests import closed_form as cf

pytestmark = pytest.mark.gpu
COUNT, SUM, AVG, MIN, MAX = 0, 1, 2, 3, 4


@pytest.fixture(scope="module")
def ops(gpu):
    from computeql_gb300 import ops as o
    return o


def host_join(build, probe, left=False):
    order = np.argsort(build, kind="stable")
    sb = build[order]
    lo = np.searchsorted(sb, probe, side="left")
    hi = np.searchsorted(sb, probe, side="right")
    pairs = []
    for p in range(len(probe)):
        if hi[p] > lo[p]:
            for j in range(lo[p], hi[p]):
                pairs.append((p, order[j]))
        elif left:
            pairs.append((p, 0xFFFFFFFF))
    return np.array(sorted(pairs), dtype=np.uint32).reshape(-1, 2)


@pytest.mark.parametrize("left", [False, True])
@pytest.mark.parametrize("dtype", [np.uint32, np.int32, np.float64])
def test_numeric_join_pairs(ops, left, dtype):
    rng = np.random.default_rng(3)
    build = rng.integers(-50, 2000, 5000).astype(dtype)   # duplicates included
    probe = rng.integers(-100, 2500, 20000).astype(dtype)
    n, pairs = ops.hash_join(ops.Column.from_numpy(build), ops.Column.from_numpy(probe), left=left)
    want = host_join(build, probe, left)
    assert n == len(want)
    assert np.array_equal(pairs, want)


def test_string_join_pairs(ops):
    rng = np.random.default_rng(4)
    words = [f"k{i:04d}" for i in range(300)] + ["", "a" * 30]
    build = [words[i] for i in rng.integers(0, len(words), 400)]
    probe = [words[i] for i in rng.integers(0, len(words), 3000)] + ["missing"]
    n, pairs = ops.hash_join(ops.StringColumn(build), ops.StringColumn(probe), left=True)
    b = np.array(build, dtype=object)
    want = []
    for p, key in enumerate(probe):
        hits = np.nonzero(b == key)[0]
        if len(hits):
            want += [(p, int(h)) for h in hits]
        else:
            want.append((p, 0xFFFFFFFF))
    assert n == len(want)
    assert np.array_equal(pairs, np.array(sorted(want), dtype=np.uint32))


def test_output_grows_past_the_first_guess(ops):
    # every probe row matches 10 build rows: 10x the max(probe, build) + probe first guess
    build = np.repeat(np.arange(100, dtype=np.uint32), 10)
    probe = np.tile(np.arange(100, dtype=np.uint32), 50)
    n, pairs = ops.hash_join(ops.Column.from_numpy(build), ops.Column.from_numpy(probe))
    assert n == 5000 * 10
    assert np.array_equal(pairs, host_join(build, probe))


@pytest.mark.parametrize("n", [1_000_000, 3_000_017])
def test_closed_form_filtered_join_to_the_50_row_table(ops, n):
    _, region, amount, _ = oracle.closed_form(n)
    regions_k = np.arange(50, dtype=np.uint32)
    zone = regions_k // 10
    dim_rows = np.nonzero(zone == 2)[0]
    res = ops.join_aggregate(ops.Column.from_numpy(region), [COUNT, SUM], [None, ops.Column.from_numpy(amount)], regions_k,
                             dim_rows=dim_rows)
    assert res["strategy"] == 1  # region has a small range: the dense path
    assert res["groups"] == 1
    assert [res["results"][0, 0], res["results"][0, 1]] == [float(x) for x in cf.join_zone_expected(n)]


def test_closed_form_join_to_the_1m_row_table(ops):
    n = 2_000_000
    _, _, _, needle = oracle.closed_form(n)
    j = np.arange(1_000_000, dtype=np.uint64)
    big_key = ((j * (n // 1_000_000)) * cf.KEY_MULTIPLIER & 0xFFFFFFFF).astype(np.uint32)
    weight = (j % 100).astype(np.float64)
    res = ops.join_aggregate(ops.Column.from_numpy(needle), [COUNT, SUM], [None, None], big_key, dim_args=[None, weight])
    assert res["strategy"] == 2  # needle_key spans the 32-bit range: the probe path
    assert [res["results"][0, 0], res["results"][0, 1]] == [1_000_000.0, cf.weight_sum(1_000_000)]


def test_c2_joins_at_10m_rows(ops):
    from computeql_gb300 import workloads
    n = 10_000_000
    t = workloads.fact_table(n)
    h = workloads.fact_numpy(n, gen=oracle.splitmix_u32)
    # dim50: k = 0..49, name_id = draw % 10, val = draw (seed 1); dim1M: k = 0..999999, seg = draw % 20 (seed 2)
    name_id = oracle.splitmix_u32(50, 1, 2, 0, 10)
    seg = oracle.splitmix_u32(1_000_000, 2, 1, 0, 20)
    # SELECT COUNT(*), SUM(amount) FROM fact JOIN dim50 ON region = k WHERE name_id = 3
    rows3 = np.nonzero(name_id == 3)[0]
    res = ops.join_aggregate(t.region, [COUNT, SUM], [None, t.amount], np.arange(50, dtype=np.uint32), dim_rows=rows3)
    sel = np.isin(h["region"], rows3)
    assert res["results"][0, 0] == sel.sum()
    assert res["results"][0, 1] == float(h["amount"][sel].astype(np.int64).sum())
    # SELECT seg, SUM(amount) FROM fact JOIN dim1M ON amount = k GROUP BY seg
    res = ops.join_aggregate(t.amount, [SUM, COUNT], [t.amount, None], np.arange(1_000_000, dtype=np.uint32),
                             group_values=[seg.astype(np.float64)])
    got = {int(seg[r]): (res["results"][g, 0], res["results"][g, 1]) for g, r in enumerate(res["dim_row"])}
    s = seg[h["amount"]]
    for v in range(20):
        m = s == v
        if m.any():
            assert got[v] == (float(h["amount"][m].astype(np.int64).sum()), float(m.sum()))


def test_dense_and_probe_paths_agree(ops):
    rng = np.random.default_rng(9)
    n = 1_000_000
    key = rng.integers(0, 5000, n).astype(np.uint32)
    v = rng.integers(-1000, 1000, n).astype(np.int32)
    dim_keys = rng.permutation(6000).astype(np.uint32)
    grp = (np.arange(6000) % 7).astype(np.float64)
    kc, vc = ops.Column.from_numpy(key), ops.Column.from_numpy(v)
    a = ops.join_aggregate(kc, [COUNT, SUM, MIN, MAX, AVG], [None, vc, vc, vc, vc], dim_keys, group_values=[grp], strategy=1)
    b = ops.join_aggregate(kc, [COUNT, SUM, MIN, MAX, AVG], [None, vc, vc, vc, vc], dim_keys, group_values=[grp], strategy=2)
    assert (a["strategy"], b["strategy"]) == (1, 2)
    ga = {grp[r]: tuple(a["results"][g]) for g, r in enumerate(a["dim_row"])}
    gb = {grp[r]: tuple(b["results"][g]) for g, r in enumerate(b["dim_row"])}
    assert ga == gb
    for gval, r in ga.items():
        keys_in = dim_keys[grp == gval]
        m = np.isin(key, keys_in)
        assert r[0] == m.sum() and r[1] == float(v[m].astype(np.int64).sum())
        assert (r[2], r[3]) == (float(v[m].min()), float(v[m].max()))


def _join_reference(ops, kc, funcs, args, dim_keys, **kw):
    """The probe path's answer (strategy 2) as {dim_row: results} in output order."""
    r = ops.join_aggregate(kc, funcs, args, dim_keys, strategy=2, **kw)
    return list(r["dim_row"]), r["results"]


@pytest.mark.parametrize("signed", [False, True])
def test_lookup_table_join_equals_the_probe(ops, signed):
    """Strategy 3 (a lookup table over a 1M-value key range) against the probe path: the same groups in
    the same order (their first kept dim row), the same COUNT/SUM/AVG/MIN/MAX."""
    rng = np.random.default_rng(21 + signed)
    n, d = 3_000_000, 1_000_000
    base = -500_000 if signed else 0
    key = (rng.integers(0, d, n) + base).astype(np.int32 if signed else np.uint32)
    v = rng.integers(-2000, 2000, n).astype(np.int32)
    dim_keys = (rng.permutation(d) + base).astype(np.int32 if signed else np.uint32).view(np.uint32)
    seg = rng.integers(0, 20, d).astype(np.float64)
    kc, vc = ops.Column.from_numpy(key), ops.Column.from_numpy(v)
    funcs, args = [COUNT, SUM, AVG, MIN, MAX], [None, vc, vc, vc, vc]
    auto = ops.join_aggregate(kc, funcs, args, dim_keys, group_values=[seg])
    assert auto["strategy"] == 3
    rows, res = _join_reference(ops, kc, funcs, args, dim_keys, group_values=[seg])
    assert list(auto["dim_row"]) == rows
    np.testing.assert_array_equal(auto["results"], res)
    # against the oracle: the joined rows per segment; and each segment's SUM from the fact side
    counts, _ = oracle.join_aggregate(key.view(np.uint32), None, dim_keys, seg.astype(np.uint32), 20)
    seg_of_key = np.empty(d, dtype=np.int64)
    seg_of_key[dim_keys.view(key.dtype).astype(np.int64) - base] = seg.astype(np.int64)
    fact_seg = seg_of_key[key.astype(np.int64) - base]
    for g, r in enumerate(auto["dim_row"]):
        s = int(seg[r])
        m = fact_seg == s
        assert auto["results"][g, 0] == counts[s] == m.sum()
        assert auto["results"][g, 1] == float(v[m].astype(np.int64).sum())


def test_lookup_table_join_with_a_dim_filter_and_no_group(ops):
    rng = np.random.default_rng(33)
    n, d = 2_000_000, 400_000
    key = rng.integers(0, d, n).astype(np.uint32)
    dim_keys = rng.permutation(d).astype(np.uint32)
    kept = np.sort(rng.choice(d, d // 3, replace=False)).astype(np.uint64)
    kc = ops.Column.from_numpy(key)
    a = ops.join_aggregate(kc, [COUNT], [None], dim_keys, dim_rows=kept, strategy=3)
    b = ops.join_aggregate(kc, [COUNT], [None], dim_keys, dim_rows=kept, strategy=2)
    assert a["strategy"] == 3 and a["groups"] == b["groups"] == 1
    assert list(a["dim_row"]) == list(b["dim_row"])
    assert a["results"][0, 0] == np.isin(key, dim_keys[kept.astype(np.int64)]).sum()
    seg = (np.arange(d) % 11).astype(np.float64)
    a = ops.join_aggregate(kc, [COUNT], [None], dim_keys, dim_rows=kept, group_values=[seg], strategy=3)
    b = ops.join_aggregate(kc, [COUNT], [None], dim_keys, dim_rows=kept, group_values=[seg], strategy=2)
    assert list(a["dim_row"]) == list(b["dim_row"])
    np.testing.assert_array_equal(a["results"], b["results"])


@pytest.mark.parametrize("signed", [False, True])
def test_lookup_table_reads_resident_dim_columns(ops, signed):
    """The lookup-table join with the dim table's key and group columns resident (dim_key_col, dim_group_col):
    nothing uploaded, the group range from the group column's zone (a superset of the kept rows' range); the
    same groups in the same order and the same totals as with host arrays, with and without a dim filter."""
    rng = np.random.default_rng(55 + signed)
    n, d = 2_000_000, 600_000
    key = rng.integers(0, d, n).astype(np.uint32)
    v = rng.integers(-3000, 3000, n).astype(np.int32)
    dim_keys = rng.permutation(d).astype(np.uint32)
    seg_i = (rng.integers(-7, 13, d) if signed else rng.integers(0, 20, d)).astype(np.int32 if signed else np.uint32)
    seg = seg_i.astype(np.float64)
    kept = np.sort(rng.choice(d, d // 2, replace=False)).astype(np.uint64)
    kc, vc = ops.Column.from_numpy(key), ops.Column.from_numpy(v)
    dk_col, seg_col = ops.Column.from_numpy(dim_keys), ops.Column.from_numpy(seg_i)
    funcs, args = [COUNT, SUM, MIN, MAX], [None, vc, vc, vc]
    for rows in (None, kept):
        host = ops.join_aggregate(kc, funcs, args, dim_keys, dim_rows=rows, group_values=[seg], strategy=3)
        dev = ops.join_aggregate(kc, funcs, args, dim_keys, dim_rows=rows, group_values=[seg], strategy=3, dim_key_col=dk_col,
                                 dim_group_col=seg_col)
        assert host["strategy"] == dev["strategy"] == 3
        assert list(dev["dim_row"]) == list(host["dim_row"])
        np.testing.assert_array_equal(dev["results"], host["results"])


def test_lookup_table_gives_way_to_repeated_dim_keys(ops):
    """Repeated dim keys: the lookup table gives way; past the dense range the probe path refuses them as
    it did before (each key must name one dim row), and a forced lookup table refuses too."""
    rng = np.random.default_rng(44)
    n, d = 1_000_000, 200_000
    key = rng.integers(0, d, n).astype(np.uint32)
    dim_keys = rng.integers(0, d, d).astype(np.uint32)
    seg = (np.arange(d) % 5).astype(np.float64)
    kc = ops.Column.from_numpy(key)
    for strategy in (0, 2, 3):
        with pytest.raises(ops.OpError):
            ops.join_aggregate(kc, [COUNT], [None], dim_keys, group_values=[seg], strategy=strategy)
    # within the dense range the repeats are joined once per dim row
    small = (key % 1000).astype(np.uint32)
    dk = rng.integers(0, 1000, 3000).astype(np.uint32)
    sg = (np.arange(3000) % 5).astype(np.float64)
    r = ops.join_aggregate(ops.Column.from_numpy(small), [COUNT], [None], dk, group_values=[sg])
    assert r["strategy"] == 1
    per_key = np.bincount(small, minlength=1000)
    for g, row in enumerate(r["dim_row"]):
        want = sum(int(per_key[k]) for k in dk[sg == sg[row]])
        assert r["results"][g, 0] == want


@pytest.mark.parametrize("dim, funcs", [(50, "sum_min_max"), (1000, "count_sum"), (1000, "sum_min_max"), (3000, "count_sum"),
                                        (16, "count_sum"), (4096, "count_sum"), (4096, "sum_min_max"), (8000, "count_sum"),
                                        (40000, "count_sum")])
def test_small_build_side_probe(ops, dim, funcs):
    """The probe (strategy 2) with a small dim table: tables that fit take the shared-memory form (the table
    and Bloom words staged by bulk copies, per-slot totals in shared memory), tables up to 16384 slots whose
    totals alone fit keep the totals there and read the table from L2, larger ones the global form;
    per dim row COUNT/SUM/MIN/MAX equal numpy's over the fact rows whose key is that row's key, with misses,
    a dim-side filter and signed arguments."""
    rng = np.random.default_rng(100 + dim)
    n = 2_000_000
    dim_keys = rng.choice(1 << 31, dim, replace=False).astype(np.uint32) * 2 + 1
    miss = rng.integers(0, 1 << 31, n).astype(np.uint32) * 2          # even: never a dim key
    key = np.where(rng.random(n) < 0.8, dim_keys[rng.integers(0, dim, n)], miss).astype(np.uint32)
    v = rng.integers(-50_000, 50_000, n).astype(np.int32)
    kept = np.sort(rng.choice(dim, max(1, dim * 3 // 4), replace=False)).astype(np.uint64)
    row_id = np.arange(dim, dtype=np.float64)                           # one group per dim row
    kc, vc = ops.Column.from_numpy(key), ops.Column.from_numpy(v)
    if funcs == "count_sum":
        fs, args = [COUNT, SUM], [None, vc]
    else:
        fs, args = [SUM, MIN, MAX], [vc, vc, vc]
    r = ops.join_aggregate(kc, fs, args, dim_keys, dim_rows=kept, group_values=[row_id], strategy=2)
    assert r["strategy"] == 2
    got = {int(row): r["results"][g] for g, row in enumerate(r["dim_row"])}
    order = np.argsort(key, kind="stable")
    sk = key[order]
    for d in kept.astype(np.int64):
        lo, hi = np.searchsorted(sk, dim_keys[d]), np.searchsorted(sk, dim_keys[d], side="right")
        vals = v[order[lo:hi]].astype(np.int64)
        if len(vals) == 0:
            assert d not in got
            continue
        want = [float(len(vals)), float(vals.sum())] if funcs == "count_sum" else [float(vals.sum()), float(vals.min()), float(vals.max())]
        assert list(got[int(d)]) == want, d
    assert list(r["dim_row"]) == sorted(got)                                # groups in dim-row order


@pytest.mark.parametrize("case", ["dim1m_by_seg", "dim50_filtered", "signed_all_funcs", "no_match_rows"])
def test_device_dim_pass_equals_the_host_pass(ops, case):
    """A dense join over a dim table resident on the device runs its dim-row pass on the device
    (cql_join_dim_fold): the same groups, in the same order (first kept dim row), the same results as the
    host pass over the host arrays of the same dim table."""
    rng = np.random.default_rng({"dim1m_by_seg": 1, "dim50_filtered": 2, "signed_all_funcs": 3, "no_match_rows": 4}[case])
    n = 3_000_000
    if case == "dim1m_by_seg":
        key = rng.integers(0, 10_000, n).astype(np.uint32)
        dk = np.arange(1_000_000, dtype=np.uint32)
        seg = rng.integers(0, 20, len(dk)).astype(np.uint32)
        funcs, fargs, dim_rows = [SUM, COUNT], ["v", None], None
    elif case == "dim50_filtered":
        key = rng.integers(0, 50, n).astype(np.uint32)
        dk = np.arange(50, dtype=np.uint32)
        seg = None
        funcs, fargs, dim_rows = [COUNT, SUM], [None, "v"], np.nonzero(rng.integers(0, 10, 50) == 3)[0]
    elif case == "signed_all_funcs":
        key = rng.integers(-3000, 3000, n).astype(np.int32)
        dk = rng.permutation(np.arange(-4000, 4000, dtype=np.int32)).view(np.uint32)
        seg = rng.integers(-7, 7, len(dk)).astype(np.int32)
        funcs, fargs, dim_rows = [COUNT, SUM, AVG, MIN, MAX], [None, "v", "v", "v", "v"], np.sort(rng.choice(len(dk), 5000, replace=False))
    else:
        key = rng.integers(0, 1000, n).astype(np.uint32)
        dk = np.arange(5000, 7000, dtype=np.uint32)          # no dim key meets a fact key
        seg = rng.integers(0, 3, len(dk)).astype(np.uint32)
        funcs, fargs, dim_rows = [COUNT, SUM], [None, "v"], None
    v = rng.integers(-100_000, 100_000, n).astype(np.int32)
    kc, vc = ops.Column.from_numpy(key), ops.Column.from_numpy(v)
    args = [vc if a == "v" else None for a in fargs]
    gvals = [seg.astype(np.float64)] if seg is not None else []
    host = ops.join_aggregate(kc, funcs, args, dk, dim_rows=dim_rows, group_values=gvals)
    dkc = ops.Column.from_numpy(dk.view(key.dtype))
    dgc = ops.Column.from_numpy(seg) if seg is not None else None
    dev = ops.join_aggregate(kc, funcs, args, dk, dim_rows=dim_rows, group_values=gvals, dim_key_col=dkc, dim_group_col=dgc)
    assert host["strategy"] == dev["strategy"] == 1
    assert dev["groups"] == host["groups"]
    assert np.array_equal(dev["dim_row"], host["dim_row"])
    assert np.array_equal(dev["results"], host["results"])
