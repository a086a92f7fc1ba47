"""The oracle against the reference's own SQLite (CPU only).

The reference's benchmarks check their answers against SQLite's over the same rows
(src/tests/bench_common.h:590-670; the tables loaded as src/tests/scale/bench_query_xlarge.c:287-340). Here
the reference's vendored amalgamation (src/third_party/sqlite/sqlite3.c) is compiled from the reference's
tree into oracle/_ref/ and answers the bench suite's SQL over the seed-0 table, the batched configuration's
drawn WHERE shapes, ORDER BY with ties and a 100k-group GROUP BY; the oracle's restatement of the reference's
operators must give the same answers - integers equal, f64 sums within 1e-12. Skipped where the reference's
tree is absent.
"""
import math

import numpy as np
import pytest

import oracle
from oracle import ref_sqlite

pytestmark = pytest.mark.skipif(not ref_sqlite.available(), reason="the reference's SQLite source is not present")
ROWS = 200_003
COUNT, SUM = 0, 1


@pytest.fixture(scope="module")
def db():
    from computeql_gb300 import workloads
    h = workloads.fact_numpy(ROWS, gen=oracle.splitmix_u32)
    d50 = {"k": np.arange(50, dtype=np.uint32), "name_id": oracle.splitmix_u32(50, workloads.DIM50_SEED, 2, 0, 10)}
    dseg = {"k": np.arange(10_000, dtype=np.uint32), "seg": oracle.splitmix_u32(1_000_000, workloads.DIM1M_SEED, 1, 0, 20)[:10_000]}
    d = ref_sqlite.Database()
    d.load("fact", {"id": np.arange(ROWS), "region": h["region"], "amount": h["amount"], "flag": h["flag"]})
    d.load("dim50", d50)
    d.load("dimseg", dseg)     # dim1M's rows 0..9999: every fact amount (< 10000) joins one of them
    yield d, h, d50, dseg
    d.close()


def test_suite_aggregates_and_filters(db):
    d, h, _, _ = db
    (s, mn, mx), = d.query("SELECT SUM(amount), MIN(amount), MAX(amount) FROM fact")
    assert (float(s), float(mn), float(mx)) == oracle.aggregate_global_cpu(h["amount"])
    (c,), = d.query("SELECT COUNT(*) FROM fact WHERE flag < 2")
    assert c == oracle.scan_and([(h["flag"], 1, 2)], ROWS)[0]
    rows = [r for (r,) in d.query("SELECT id FROM fact WHERE flag < 2 AND amount >= 5000 ORDER BY id")]
    assert rows == list(oracle.scan_and([(h["flag"], 1, 2), (h["amount"], 4, 5000)], ROWS, want_rows=True)[1])


def test_suite_group_bys(db):
    d, h, _, _ = db
    want = d.query("SELECT region, SUM(amount), COUNT(*) FROM fact GROUP BY region ORDER BY region")
    counts, sums, _, _ = oracle.group_dense(h["region"], 0, 50, [SUM, COUNT], [h["amount"], None])
    assert want == [(g, int(sums[g, 0]), int(counts[g])) for g in range(50) if counts[g]]
    want = d.query("SELECT amount, COUNT(*), SUM(region), MIN(region), MAX(region) FROM fact GROUP BY amount ORDER BY amount")
    counts, sums, mins, maxs = oracle.group_dense(h["amount"], 0, 10_000, [COUNT, SUM, 3, 4], [None, h["region"], h["region"], h["region"]])
    assert want == [(a, int(counts[a]), int(sums[a, 1]), int(mins[a, 2]), int(maxs[a, 3])) for a in range(10_000) if counts[a]]


def test_suite_joins(db):
    d, h, d50, dseg = db
    (c, s), = d.query("SELECT COUNT(*), SUM(f.amount) FROM fact f JOIN dim50 d ON f.region = d.k WHERE d.name_id = 3")
    keep = np.where(d50["name_id"] == 3, 0, 0xFFFFFFFF).astype(np.uint32)
    ec, es = oracle.join_aggregate(h["region"], h["amount"], d50["k"], keep, 1)
    assert (c, s or 0) == (int(ec[0]), int(es[0]))
    want = d.query("SELECT d.seg, SUM(f.amount), COUNT(*) FROM fact f JOIN dimseg d ON f.amount = d.k GROUP BY d.seg ORDER BY d.seg")
    ec, es = oracle.join_aggregate(h["amount"], h["amount"], dseg["k"], dseg["seg"], 20)
    assert want == [(g, int(es[g]), int(ec[g])) for g in range(20) if ec[g]]


def test_order_by_with_ties_by_position(db):
    d, h, _, _ = db
    got = [r - 1 for (r,) in d.query("SELECT rowid FROM fact ORDER BY amount DESC, region, rowid")]
    assert got == list(oracle.sort_rows([h["amount"], h["region"]], desc=[1, 0]).astype(np.int64))


def test_hash_group_by_100k_keys(db):
    d, h, _, _ = db
    key = (h["amount"].astype(np.uint64) * 50 + h["region"]).astype(np.uint32)     # 500k possible values
    d.execute("CREATE TABLE hk AS SELECT amount * 50 + region AS k, flag FROM fact")
    want = d.query("SELECT k, COUNT(*), SUM(flag), MIN(flag), MAX(flag) FROM hk GROUP BY k ORDER BY k")
    keys, counts, sums, mins, maxs = oracle.group_cpu_reduce(key, [h["flag"]], 400_000)
    order = np.argsort(keys)
    got = [(int(keys[i]), int(counts[i]), int(sums[i, 0]), int(mins[i, 0]), int(maxs[i, 0])) for i in order]
    assert got == want


def test_batched_where_shapes(db):
    """The batched configuration's drawn WHERE shapes (AND/OR chains over u32 and f64 columns): the oracle's
    interpreter and its batch evaluator against SQLite's WHERE, COUNT equal and SUM(f64) within 1e-12."""
    from computeql_gb300 import ops
    from tests.batch_workload import F64, U32, queries, table
    from tests.where_shapes import oracle_batch, oracle_mask
    n = 50_001
    arrays = table(n, 12)
    d, _, _, _ = db
    d.load("bt", arrays)
    cols = {c: ops.Column(ops.TYPE_U32, n, zone=(0.0, 65535.0)) for c in U32}
    cols.update({c: ops.Column(ops.TYPE_F64, n) for c in F64})
    qs = queries(64, 29, 5)
    progs = [ops.Program(w, cols) for w, _ in qs]
    counts, sums = oracle_batch(progs, [s for _, s in qs], arrays, n)
    for i, (w, s) in enumerate(qs):
        sql = to_sql(w)
        (c, total), = d.query(f"SELECT COUNT(*), TOTAL({s}) FROM bt WHERE {sql}")
        assert c == counts[i] == oracle_mask(progs[i], arrays).sum(), (w, sql)
        assert math.isclose(total, sums[i], rel_tol=1e-12, abs_tol=0.0) or total == sums[i], (w, total, sums[i])


def to_sql(sexpr):
    """The test's s-expression WHERE as SQL (the same comparisons, AND/OR with explicit parentheses)."""
    toks = sexpr.replace("(", " ( ").replace(")", " ) ").split()
    pos = 0

    def parse():
        nonlocal pos
        t = toks[pos]
        if t != "(":
            pos += 1
            return t
        pos += 1
        op = toks[pos]
        pos += 1
        args = []
        while toks[pos] != ")":
            args.append(parse())
        pos += 1
        if op in ("and", "or"):
            return "(" + f" {op.upper()} ".join(args) + ")"
        sym = {"=": "=", "!=": "<>", "<": "<", "<=": "<=", ">": ">", ">=": ">="}[op]
        return f"({args[0]} {sym} {args[1]})"
    return parse()
