"""Streamed operators over the resident chunk cache (GB300 only).

The reference streams its big operators in chunks through its resident cache: the scan
(qe_scan_filter_streamed, src/query_exec/query_exec.c:2242-2494), the dense group-by
(qe_aggregate_dense_streamed, :7984-8068), the fact side of the join-aggregate (qe_join_probe_stream_core,
:8080-8420) and the global aggregate (:8842-9112). Here each runs over host columns:

* with a cache budget smaller than the table (chunks evicted as later ones arrive), the answers equal the
  resident operators' over the same columns held whole in HBM, bit for bit;
* with a budget that holds the table, a second pass uploads nothing; with the small budget it uploads again
  and the cache's evictions rise;
* the streamed f64 global aggregate adds every workgroup partial of every chunk into one running sum (the
  reference's fold order): it equals replaying that fold through cqlcuda's accumulate entry point chunk by
  chunk over device copies, bit for bit, and is within 1e-12 of a compensated sum.
"""
import ctypes as C

import numpy as np
import pytest

import oracle

pytestmark = pytest.mark.gpu
COUNT, SUM, AVG, MIN, MAX = 0, 1, 2, 3, 4
N = 6_000_011
CHUNK = 1 << 20


@pytest.fixture(scope="module")
def env(gpu):
    from computeql_gb300 import native, ops
    rng = np.random.default_rng(41)
    t = {"region": rng.integers(0, 50, N).astype(np.uint32), "amount": rng.integers(0, 10_000, N).astype(np.uint32),
         "flag": rng.integers(0, 100, N).astype(np.uint32), "delta": rng.integers(-5000, 5000, N).astype(np.int32)}
    dev = {k: ops.Column.from_numpy(v) for k, v in t.items()}
    return ops, native, native.load_ops(), t, dev


def host_col(native, uid, arr, zone=True):
    types = {np.dtype(np.uint32): 1, np.dtype(np.int32): 7, np.dtype(np.float64): 4}
    h = native.CqlHostColumn()
    h.uid, h.generation, h.values, h.type = uid, 1, arr.ctypes.data, types[arr.dtype]
    h.has_range = 1 if zone else 0
    h.zone_min, h.zone_max = (float(arr.min()), float(arr.max())) if zone else (0.0, 0.0)
    return h


def cache(lib, budget):
    c = lib.cqlops_resident_create(budget, None)
    assert c
    return c


SMALL = 3 * CHUNK * 4 + 1024     # three 4 MB chunks: a 24 MB column does not fit


@pytest.mark.parametrize("budget", [SMALL, 0])
def test_streamed_scan_equals_the_resident_scan(env, budget):
    ops, native, lib, t, dev = env
    cols = (native.CqlHostColumn * 2)(host_col(native, 1, t["flag"]), host_col(native, 2, t["amount"]))
    leaves = (native.CqlLeaf * 2)(native.CqlLeaf(0, ops.CMP_LT, 3.0), native.CqlLeaf(1, ops.CMP_GE, 9000.0))
    want_n, want_rows = ops.scan_simple([dev["flag"], dev["amount"]], [(0, ops.CMP_LT, 3), (1, ops.CMP_GE, 9000)], want_rows=True)
    c = cache(lib, budget)
    uploads = []
    for _ in range(2):
        cnt, up = C.c_uint64(), C.c_uint64()
        rows = np.zeros(N, dtype=np.uint32)
        assert lib.cqlops_scan_simple_streamed(c, cols, 2, N, leaves, 2, CHUNK, C.byref(cnt), native.ptr(rows), N, C.byref(up)), \
            native.last_error()
        assert cnt.value == want_n and np.array_equal(rows[: cnt.value], want_rows)
        uploads.append(up.value)
    assert uploads[0] == 2 * N * 4
    if budget == 0:
        assert uploads[1] == 0
    else:
        # the cache keeps what fits (entries used once go newest first): the rest is uploaded again
        assert 2 * N * 4 - budget <= uploads[1] < 2 * N * 4 + 1
    st = lib.cqlops_resident_stats(c)
    if budget:
        assert st.evicted_bytes > 0 and st.bytes_in_use <= budget
    lib.cqlops_resident_destroy(c)


@pytest.mark.parametrize("budget", [SMALL, 0])
def test_streamed_dense_group_by_equals_the_resident_one(env, budget):
    ops, native, lib, t, dev = env
    funcs = [COUNT, SUM, MIN, MAX, SUM]
    want = ops.group_dense(dev["region"], funcs, [None, dev["amount"], dev["delta"], dev["delta"], dev["region"]])
    key = host_col(native, 10, t["region"])
    amount, delta = host_col(native, 11, t["amount"]), host_col(native, 12, t["delta"])
    args = (C.c_void_p * 5)(None, C.addressof(amount), C.addressof(delta), C.addressof(delta), C.addressof(key))
    fa = np.array(funcs, dtype=np.uint32)
    c = cache(lib, budget)
    for pass_ in range(2):
        g, mk, up = C.c_uint64(), C.c_int64(), C.c_uint64()
        counts = np.zeros(50, dtype=np.uint64)
        sums, mins, maxs = (np.zeros(50 * 5, dtype=np.int64) for _ in range(3))
        assert lib.cqlops_group_dense_streamed(c, C.byref(key), N, 5, native.ptr(fa), args, CHUNK, 50, C.byref(g), C.byref(mk),
                                               native.ptr(counts), native.ptr(sums), native.ptr(mins), native.ptr(maxs), C.byref(up)), \
            native.last_error()
        assert mk.value == want[0] and g.value == len(want[1])
        assert np.array_equal(counts, want[1])
        assert np.array_equal(sums.reshape(50, 5)[:, [1, 4]], want[2][:, [1, 4]])
        assert np.array_equal(mins.reshape(50, 5)[:, 2], want[3][:, 2]) and np.array_equal(maxs.reshape(50, 5)[:, 3], want[4][:, 3])
        if pass_ == 1:
            assert up.value == 0 if budget == 0 else 3 * N * 4 - budget <= up.value <= 3 * N * 4
    lib.cqlops_resident_destroy(c)


@pytest.mark.parametrize("strategy", [1, 2])
def test_streamed_join_equals_the_resident_join(env, strategy):
    """The dim1M-style join grouped by a dim value: the fact key and the summed column streamed."""
    ops, native, lib, t, dev = env
    dk = np.arange(20_000, dtype=np.uint32)
    seg = (np.arange(20_000) * 7 % 20).astype(np.float64)
    funcs = [SUM, COUNT, MIN, MAX, AVG]
    want = ops.join_aggregate(dev["amount"], funcs, [dev["delta"], None, dev["delta"], dev["delta"], dev["delta"]], dk,
                              group_values=[seg], strategy=strategy)
    key, delta = host_col(native, 20, t["amount"]), host_col(native, 21, t["delta"])
    fargs = (C.c_void_p * 5)(C.addressof(delta), None, C.addressof(delta), C.addressof(delta), C.addressof(delta))
    fa = np.array(funcs, dtype=np.uint32)
    segs = (C.c_void_p * 1)(seg.ctypes.data)
    q = native.CqlJoinAgg(None, 5, fa.ctypes.data, None, None, dk.ctypes.data, len(dk), None, 0, 1, C.addressof(segs), strategy)
    c = cache(lib, SMALL)
    groups, strat, up = C.c_uint64(), C.c_uint32(), C.c_uint64()
    dim_row = np.zeros(len(dk), dtype=np.uint64)
    res = np.zeros(len(dk) * 5, dtype=np.float64)
    assert lib.cqlops_join_aggregate_streamed(c, C.byref(q), C.byref(key), fargs, N, CHUNK, len(dk), C.byref(groups), native.ptr(dim_row),
                                              native.ptr(res), C.byref(strat), C.byref(up)), native.last_error()
    g = groups.value
    assert strat.value == strategy and g == want["groups"]
    assert np.array_equal(dim_row[:g], want["dim_row"])
    assert np.array_equal(res[: g * 5].reshape(g, 5), want["results"])
    assert up.value == 2 * N * 4
    lib.cqlops_resident_destroy(c)


def test_streamed_f64_aggregate_folds_every_partial_in_order(env):
    ops, native, lib, _, _ = env
    rng = np.random.default_rng(42)
    n = 5_000_003
    host = rng.lognormal(3.0, 1.0, n) * np.where(rng.random(n) < 0.3, -1.0, 1.0)
    c = cache(lib, SMALL * 2)
    s, mn, mx, up = C.c_double(), C.c_double(), C.c_double(), C.c_uint64()
    assert lib.cqlops_aggregate_global_streamed(c, 30, 1, host.ctypes.data, ops.TYPE_F64, n, CHUNK, C.byref(s), C.byref(mn), C.byref(mx),
                                                C.byref(up)), native.last_error()
    # the same fold replayed: every chunk's partials added into one running total, chunk by chunk
    rs, rmn, rmx = C.c_double(0.0), C.c_double(1.7976931348623157e308), C.c_double(-1.7976931348623157e308)
    for first in range(0, n, CHUNK):
        col = ops.Column.from_numpy(host[first: first + CHUNK])
        arr = (native.CqlColumn * 1)(col.c())
        assert lib.cqlops_aggregate_global_accumulate(arr, 1, C.byref(rs), C.byref(rmn), C.byref(rmx))
    assert (s.value, mn.value, mx.value) == (rs.value, rmn.value, rmx.value)
    exact = oracle.compensated_sum(host)
    assert abs(s.value - exact) <= 1e-12 * max(abs(exact), np.abs(host).sum() * 1e-3)
    assert (mn.value, mx.value) == (float(host.min()), float(host.max()))
    # an empty column gives the fold's starting sentinels, as the reference's does
    assert lib.cqlops_aggregate_global_streamed(c, 31, 1, host.ctypes.data, ops.TYPE_F64, 0, CHUNK, C.byref(s), C.byref(mn), C.byref(mx),
                                                None)
    assert (s.value, mn.value, mx.value) == (0.0, 1.7976931348623157e308, -1.7976931348623157e308)
    lib.cqlops_resident_destroy(c)
