"""The batched shared scan (cqlops_batch_filter_aggregate) against the oracle, query by query.

Every query of a batch must give alone what the oracle gives: the count of rows its condition
matches (the oracle's restatement of the bytecode interpreter) bit for bit, and its SUM within 1e-12
of the exact sum of those rows (math.fsum). The workload is the batched configuration's table shape
(4 u32 + 4 f64 columns) with shapes drawn as the reference's per-query kernel benchmark draws them.
"""
import math

import numpy as np
import pytest

from tests.batch_workload import F64, U32, queries, table
from tests.where_shapes import oracle_mask

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def ops(gpu):
    from computeql_gb300 import ops as o
    return o


def _columns(ops, arrays):
    return {n: ops.Column.from_numpy(a) for n, a in arrays.items()}


def _check(ops, arrays, cols, qs, rows_per_thread=8):
    progs = [ops.Program(where, cols) for where, _ in qs]
    counts, sums, shapes = ops.batch_aggregate(progs, [s for _, s in qs], rows_per_thread)
    for i, (where, scol) in enumerate(qs):
        m = oracle_mask(progs[i], arrays).astype(bool)
        assert counts[i] == m.sum(), where
        if scol is None:
            continue
        exact = math.fsum(arrays[scol][m])
        assert abs(sums[i] - exact) <= 1e-12 * max(abs(exact), 1e-300), (where, sums[i], exact)
    return shapes


@pytest.mark.parametrize("rows_per_thread", [0, 4, 8, 16])
def test_batch_matches_each_query_alone(ops, rows_per_thread):
    arrays = table(2_000_003, 1)
    cols = _columns(ops, arrays)
    qs = queries(64, 8, 7)
    shapes = _check(ops, arrays, cols, qs, rows_per_thread)
    assert shapes <= 8


@pytest.mark.parametrize("rows_per_thread", [0, 8])
def test_more_queries_than_one_launch_holds(ops, rows_per_thread):
    arrays = table(300_001, 2)
    cols = _columns(ops, arrays)
    qs = queries(500, 29, 11)
    assert _check(ops, arrays, cols, qs, rows_per_thread) <= 29


@pytest.mark.parametrize("rows_per_thread", [0, 8])
def test_count_only_and_special_values(ops, rows_per_thread):
    rng = np.random.default_rng(5)
    n = 100_000
    arrays = table(n, 3)
    d = arrays["d0"]
    d[::7] = 0.0
    d[3::7] = -0.0
    d[5::101] = np.nan
    d[6::103] = np.inf
    d[2::107] = -np.inf
    arrays["d0"] = d
    cols = _columns(ops, {**arrays, "d0": np.where(np.isnan(d), 0.0, d)})   # the summed copy has no NaN
    cols["d0"] = ops.Column.from_numpy(d)
    qs = [("(> d0 0.0)", None), ("(>= d0 0.0)", None), ("(= d0 0.0)", None), ("(!= d0 0.0)", None), ("(< d0 -0.0)", None),
          ("(<= d0 0.0)", None), ("(< d0 1e308)", None), ("(> d0 -1e308)", None), ("(and (> d0 0.25) (< d0 0.5))", "d1"),
          ("(or (= u0 7) (< u1 100))", "d2"), ("(and (>= u2 65535) (<= u2 65535))", None), ("(< u3 0)", None)]
    progs = [ops.Program(w, cols) for w, _ in qs]
    counts, sums, _ = ops.batch_aggregate(progs, [s for _, s in qs], rows_per_thread)
    for i, (w, s) in enumerate(qs):
        m = oracle_mask(progs[i], arrays).astype(bool)
        assert counts[i] == m.sum(), w
        if s:
            exact = math.fsum(arrays[s][m])
            assert abs(sums[i] - exact) <= 1e-12 * abs(exact)


@pytest.mark.parametrize("rows_per_thread", [0, 8])
def test_signed_and_float_columns(ops, rows_per_thread):
    rng = np.random.default_rng(8)
    n = 500_000
    arrays = {"i": rng.integers(-1000, 1000, n).astype(np.int32), "f": rng.normal(size=n).astype(np.float32),
              "v": rng.lognormal(3.0, 1.0, n)}
    cols = _columns(ops, arrays)
    qs = [("(< i -10)", "v"), ("(>= i 999)", "v"), ("(and (> f 0.5) (< i 0))", "v"), ("(<= f -1.25)", "i"),
          ("(or (= i 0) (> f 2.5))", "f"), ("(< f 0.1)", None)]
    progs = [ops.Program(w, cols) for w, _ in qs]
    counts, sums, _ = ops.batch_aggregate(progs, [s for _, s in qs], rows_per_thread)
    for i, (w, s) in enumerate(qs):
        m = oracle_mask(progs[i], arrays).astype(bool)
        assert counts[i] == m.sum(), w
        if s:
            exact = math.fsum(arrays[s][m].astype(np.float64))
            assert abs(sums[i] - exact) <= 1e-12 * abs(exact), w


def test_tile_and_register_forms_agree(ops):
    """The two kernel forms give identical counts; their sums differ only by the rounding of each row's
    summand at the scale each form chooses, far inside 1e-12."""
    arrays = table(50_000, 4)
    cols = _columns(ops, arrays)
    qs = queries(96, 12, 21)
    progs = [ops.Program(w, cols) for w, _ in qs]
    c0, s0, _ = ops.batch_aggregate(progs, [s for _, s in qs], 0)
    c8, s8, _ = ops.batch_aggregate(progs, [s for _, s in qs], 8)
    assert np.array_equal(c0, c8)
    for i, (w, scol) in enumerate(qs):
        if scol:
            assert abs(s0[i] - s8[i]) <= 1e-12 * max(abs(s8[i]), 1e-300), w


def test_plan_graph_replays_a_repeated_shape(ops):
    """Batches of the same shapes and query count run as one CUDA graph: the first captures it, the next
    replay it with their own literals (the uploaded thresholds); every batch's results equal the oracle's."""
    import ctypes as C
    from computeql_gb300 import native
    from tests.batch_workload import shapes
    arrays = table(1_000_003, 5)
    cols = _columns(ops, arrays)
    gens = shapes(6, 21)
    lib = native.load_cuda()

    def stats():
        c, r, f = C.c_uint64(), C.c_uint64(), C.c_uint64()
        lib.cqlcuda_graph_stats(C.byref(c), C.byref(r), C.byref(f))
        return c.value, r.value, f.value

    before = stats()
    for seed in (100, 101, 102):
        rng = np.random.default_rng(seed)
        qs = [(gens[q % 6](rng), F64[q % 4]) for q in range(24)]
        _check(ops, arrays, cols, qs)
    after = stats()
    assert after[1] - before[1] >= 1      # a later batch replayed the graph of the first
    assert after[2] == before[2]          # and no record fell back to an eager run


def test_batched_configuration_100m_rows_512_queries(ops):
    """The batched configuration at its own size: 100M rows of 4 u32 + 4 f64 columns, 512 queries over 29
    shapes, the form chosen by the autotuner. Every query's COUNT bit for bit and its SUM within 1e-12 of the
    oracle's compensated sum over the same rows (the oracle's batch evaluator, all host threads, one pass)."""
    import oracle
    from tests.where_shapes import oracle_batch
    rows = 100_000_000
    arrays = table(rows, 0)
    cols = _columns(ops, arrays)
    qs = queries(512, 29, 1)
    progs = [ops.Program(w, cols) for w, _ in qs]
    counts, sums, shapes = ops.batch_aggregate(progs, [s for _, s in qs], 0xFFFFFFFF)
    assert shapes <= 29
    for c in cols.values():
        c.buffer.close()
    oracle.set_threads(0)
    want_counts, want_sums = oracle_batch(progs, [s for _, s in qs], arrays, rows)
    assert np.array_equal(counts, want_counts)
    for i, (w, _) in enumerate(qs):
        assert abs(sums[i] - want_sums[i]) <= 1e-12 * max(abs(want_sums[i]), 1e-300), (w, sums[i], want_sums[i])
    assert 0 < int((counts > 0).sum()) and int(counts.max()) < rows     # the draws give neither all-empty nor all-full batches
