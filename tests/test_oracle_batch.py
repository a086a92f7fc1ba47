"""The oracle's batch evaluator against its row interpreter (CPU only).

orc_batch_count_sum runs the scan bytecode a block of rows at a time over every program of a batch; it
is the checker of the batched shared scan at 100M rows x 512 queries, where the row interpreter with a
mask per query would take too long. Here both run on the same seeded table and the same drawn queries:
counts equal bit for bit, sums within 1e-15 relative of the exact sum of the matching rows.
"""
import math

import numpy as np

import oracle
from computeql_gb300 import ops
from tests.batch_workload import F64, U32, queries, table
from tests.where_shapes import oracle_batch, oracle_mask


def test_batch_evaluator_equals_the_row_interpreter():
    rows = 50_003
    arrays = table(rows, 4)
    cols = {n: ops.Column(ops.TYPE_U32, rows, zone=(0.0, 65535.0)) for n in U32}
    cols.update({n: ops.Column(ops.TYPE_F64, rows) for n in F64})
    qs = queries(96, 12, 3) + [("(or (= u0 7) (< u1 100))", None), ("(and (>= u2 65535) (<= u2 65535))", "d1")]
    progs = [ops.Program(w, cols) for w, _ in qs]
    oracle.set_threads(3)
    try:
        counts, sums = oracle_batch(progs, [s for _, s in qs], arrays, rows)
    finally:
        oracle.set_threads(0)
    for i, (w, s) in enumerate(qs):
        m = oracle_mask(progs[i], arrays).astype(bool)
        assert counts[i] == m.sum(), w
        exact = math.fsum(arrays[s][m]) if s else 0.0
        assert abs(sums[i] - exact) <= 1e-15 * abs(exact), (w, sums[i], exact)
