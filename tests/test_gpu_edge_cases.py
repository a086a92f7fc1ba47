"""Empty and tiny tables through every operator (GB300 only).

The reference's operators give the empty answer for a table of no rows - no matched rows, no groups, no pairs,
sums of 0 and the fold's starting extremes (+-F64_MAX, qe_agg_stream_retire, query_exec.c:8812-8841) - and
this backend gives it without launching anything. Tables of 1, 3, 5 and 33 rows (below one 16-byte vector,
one warp, one tile) check the kernels' tails against the oracle.
"""
import numpy as np
import pytest

import oracle

pytestmark = pytest.mark.gpu
COUNT, SUM, AVG, MIN, MAX = 0, 1, 2, 3, 4
F64_MAX = 1.7976931348623157e308


@pytest.fixture(scope="module")
def ops(gpu):
    from computeql_gb300 import ops as o
    return o


def test_empty_table_gives_the_empty_answers(ops):
    lib = __import__("computeql_gb300.native", fromlist=["native"]).load_cuda()
    e32 = ops.Column.from_numpy(np.zeros(0, dtype=np.uint32))
    e64 = ops.Column.from_numpy(np.zeros(0, dtype=np.float64))
    five = ops.Column.from_numpy(np.arange(5, dtype=np.uint32))
    prog = ops.Program("(or (< a 3) (> b 0.5))", {"a": e32, "b": e64})
    progs = [ops.Program("(< a 3)", {"a": e32, "b": e64}), ops.Program("(> b 0.5)", {"a": e32, "b": e64})]
    launched = {}

    def run(name, fn):
        before = lib.cqlcuda_kernel_launch_count()
        out = fn()
        launched[name] = lib.cqlcuda_kernel_launch_count() - before
        return out

    s, mn, mx = run("aggregate_global", lambda: ops.aggregate_global([e32, e64]))
    assert list(s) == [0.0, 0.0] and list(mn) == [F64_MAX] * 2 and list(mx) == [-F64_MAX] * 2
    assert run("scan_simple", lambda: ops.scan_simple([e32], [(0, ops.CMP_LT, 5)]))[0] == 0
    cnt, rows = run("scan_simple rows", lambda: ops.scan_simple([e32], [(0, ops.CMP_GE, 0)], want_rows=True))
    assert cnt == 0 and len(rows) == 0
    for strategy in (ops.SCAN_GENERATED, ops.SCAN_INTERPRETER):
        assert run(f"scan_filter {strategy}", lambda: ops.scan_filter(prog, strategy=strategy))[0] == 0
    c, sums, mins, maxs = run("fused_aggregate", lambda: ops.fused_aggregate(prog, ["b"]))
    assert (c, sums[0], mins[0], maxs[0]) == (0.0, 0.0, F64_MAX, -F64_MAX)
    assert run("group_hash", lambda: ops.group_hash([e32], [COUNT, SUM], [None, e64]))["groups"] == 0
    counts, sums, _ = run("batch_aggregate", lambda: ops.batch_aggregate(progs, [None, "b"], 8))
    assert list(counts) == [0, 0] and list(sums) == [0.0, 0.0]
    assert len(run("sort_rows", lambda: ops.sort_rows([e32]))) == 0
    r = run("join_aggregate", lambda: ops.join_aggregate(e32, [COUNT, SUM], [None, e32], np.arange(10, dtype=np.uint32)))
    assert r["groups"] == 0
    n, pairs = run("hash_join", lambda: ops.hash_join(five, e32))
    assert n == 0
    assert {k: v for k, v in launched.items() if v} == {}     # none of the above launched a kernel


def test_empty_build_side_of_a_join(ops):
    probe = ops.Column.from_numpy(np.array([3, 1, 4, 1, 5], dtype=np.uint32))
    empty = ops.Column.from_numpy(np.zeros(0, dtype=np.uint32))
    assert ops.hash_join(empty, probe)[0] == 0
    n, pairs = ops.hash_join(empty, probe, left=True)
    assert n == 5 and pairs.tolist() == [[r, 0xFFFFFFFF] for r in range(5)]


@pytest.mark.parametrize("n", [1, 3, 5, 33])
def test_tiny_tables_against_the_oracle(ops, n):
    rng = np.random.default_rng(n)
    a = rng.integers(0, 20, n).astype(np.uint32)
    b = rng.integers(-1000, 1000, n).astype(np.int32)
    f = rng.random(n)
    ca, cb, cf_ = ops.Column.from_numpy(a), ops.Column.from_numpy(b), ops.Column.from_numpy(f)
    s, mn, mx = ops.aggregate_global([ca, cb, cf_])
    for i, arr in enumerate((a, b)):
        assert (s[i], mn[i], mx[i]) == oracle.aggregate_global_cpu(arr)
    fs, fmn, fmx = oracle.aggregate_global_cpu(f)
    assert abs(s[2] - fs) <= 1e-12 * abs(fs) and (mn[2], mx[2]) == (fmn, fmx)      # f64: the fold order may differ
    cnt, rows = ops.scan_simple([ca, cb], [(0, ops.CMP_LT, 10), (1, ops.CMP_GE, 0)], want_rows=True)
    want_cnt, want_rows = oracle.scan_and([(a, 1, 10), (b, 4, 0)], n, want_rows=True)
    assert cnt == want_cnt and list(rows) == list(want_rows)
    mk, counts, sums, mins, maxs = ops.group_dense(ca, [COUNT, SUM, MIN, MAX], [None, cb, cb, cb])
    ec, es, emn, emx = oracle.group_dense(a, mk, len(counts), [COUNT, SUM, MIN, MAX], [None, b, b, b])
    present = counts > 0
    assert np.array_equal(counts, ec) and np.array_equal(sums[:, 1], es[:, 1])
    assert np.array_equal(mins[present, 2], emn[present, 2]) and np.array_equal(maxs[present, 3], emx[present, 3])
    r = ops.group_hash([ca], [COUNT, SUM], [None, cb])
    keys = a[r["repr_row"].astype(np.int64)]
    got = sorted(zip(keys.tolist(), r["counts"].tolist(), r["results"][:, 1].tolist()))
    want = sorted((int(k), int((a == k).sum()), float(b[a == k].astype(np.int64).sum())) for k in np.unique(a))
    assert got == want
    assert list(ops.sort_rows([cb, ca], desc=[1, 0])) == list(oracle.sort_rows([b, a], desc=[1, 0]))
    dim = np.arange(20, dtype=np.uint32)
    seg = (dim % 3).astype(np.float64)
    for strategy in (1, 2):
        j = ops.join_aggregate(ca, [COUNT, SUM], [None, cb], dim, group_values=[seg], strategy=strategy)
        got = {int(seg[int(d)]): tuple(j["results"][g]) for g, d in enumerate(j["dim_row"])}
        for sgv in range(3):
            m = (a % 3) == sgv
            if m.any():
                assert got[sgv] == (float(m.sum()), float(b[m].astype(np.int64).sum())), (strategy, sgv)
    rows_sel = np.array(sorted(set(rng.integers(0, n, min(n, 4)).tolist())), dtype=np.uint32)
    vals = ops.gather_rows([ca, cb, cf_], rows=rows_sel)
    assert np.array_equal(np.asarray(vals[0]), a[rows_sel]) and np.array_equal(np.asarray(vals[1]), b[rows_sel])
    assert np.array_equal(np.asarray(vals[2]), f[rows_sel])
