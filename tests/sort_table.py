"""The ORDER BY test table of the reference's sort test, restated with numpy.

pq_load_table (src/tests/bench_query_sort.c:66-113) fills id, a u32, b i32, c u64, d f32 and e f64 from
the bench generator bench_rng_next (src/tests/bench_common.h:31-37, splitmix64 from the state
0x9E3779B97F4A7C15 advanced by the same constant before each draw), three draws per row; --narrow gives
a a 16-bit range and b a byte range. The string columns are left out: string keys sort on the CPU there.
SORT_CASES are the test's ORDER BY clauses (bench_query_sort.c:256-268) as (column, desc) lists.
"""
import numpy as np

from tests.bench_rng import GAMMA, mix as _mix, rows as _rows


def pq_table(rows, narrow=False):
    r = _rows(int(GAMMA), rows, 3)
    r0, r1, r2 = r[:, 0], r[:, 1], r[:, 2]
    hi0 = (r0 >> np.uint64(32))
    if narrow:
        a = (r0 % np.uint64(60000)).astype(np.uint32)
        b = ((hi0 % np.uint64(200)).astype(np.int64) - 100).astype(np.int32)
    else:
        a = (r0 % np.uint64(2000000)).astype(np.uint32)
        b = hi0.astype(np.uint32).view(np.int32)
    c = r1 % np.uint64(1000000000000)
    d = ((r1 >> np.uint64(40)) % np.uint64(1000)).astype(np.float32) / np.float32(1000.0)
    e = (r2 % np.uint64(100000)).astype(np.float64) / 100.0
    return {"id": np.arange(rows, dtype=np.uint32), "a": a, "b": b, "c": c, "d": d.astype(np.float32), "e": e}


SORT_CASES = [
    [("a", 0)],
    [("a", 1)],
    [("e", 0)],
    [("c", 1)],
    [("b", 0), ("a", 1)],
    [("d", 1), ("a", 0)],
    [("e", 0), ("c", 0)],
    [("c", 0), ("e", 1), ("d", 0)],
    [("c", 0), ("d", 1), ("a", 0), ("b", 1)],
    [("b", 0), ("d", 0)],
]


def verify_order(table, case, order):
    """pq_sort_verify (bench_query_sort.c:144-178): a permutation of the table with its keys in order.

    Returns 0 when it holds, else the first bad position plus one. The tie rule (equal keys keep their
    input order) is checked beside it.
    """
    n = len(table["a"])
    order = np.asarray(order, dtype=np.int64)
    if len(order) != n or order.min(initial=0) < 0 or order.max(initial=0) >= n:
        return 1
    if len(np.unique(order)) != n:
        return 1
    if n < 2:
        return 0
    undecided = np.ones(n - 1, dtype=bool)
    bad = np.zeros(n - 1, dtype=bool)
    for col, desc in case:
        v = table[col].astype(np.float64)[order]
        prev, cur = v[:-1], v[1:]
        differ = undecided & (prev != cur)
        wrong = (prev > cur) if not desc else (prev < cur)
        bad |= differ & wrong
        undecided &= ~differ
    bad |= undecided & (order[:-1] > order[1:])   # ties by input position
    hits = np.nonzero(bad)[0]
    return int(hits[0]) + 2 if len(hits) else 0
