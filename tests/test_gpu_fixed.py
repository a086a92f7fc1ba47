"""Fixed-point decimals through the C ABI against the oracle's FP64 restatement of the reference.

The kernels decide each value's scale and scale it in integer arithmetic on the double's bits; the
oracle does what the reference does in FP64 (qe_fixed_point_task, src/query_exec/query_exec.c:3893-3933,
and aggregate_dense_f64.comp:73-145). Both must agree on every value: the per-value scale of
adversarial inputs (ulp neighbours of decimals, products just off n + 0.5, powers of two, magnitudes
at 2^31, subnormals, NaN, infinities, f32 values), the column scale, and every group's COUNT, SUM,
AVG, MIN, MAX and smallest row, bit for bit.
"""
import ctypes as C

import numpy as np
import pytest

import oracle

pytestmark = pytest.mark.gpu
COUNT, SUM, AVG, MIN, MAX = 0, 1, 2, 3, 4


@pytest.fixture(scope="module")
def ops(gpu):
    from computeql_gb300 import ops as o
    return o


def adversarial_values(n, seed):
    rng = np.random.default_rng(seed)
    parts = []
    for s in range(8):
        w = rng.integers(-(2**31) // 10**min(s, 6), 2**31 // 10**min(s, 6), n // 16)
        d = w / 10.0**s
        parts += [d, np.nextafter(d, np.inf), np.nextafter(d, -np.inf)]
    parts.append(rng.normal(0, 1e4, n // 16))
    parts.append(rng.integers(0, 2**20, n // 16) * 2.0**-rng.integers(0, 40, n // 16))   # dyadic: 2^-k
    half = (rng.integers(0, 2**30, n // 16) + 0.5) / 10.0**rng.integers(0, 7, n // 16)     # products near n + 0.5
    parts += [half, np.nextafter(half, np.inf)]
    parts.append(np.array([0.0, -0.0, 1.0, -1.0, 0.5, 2.0**30, 2.0**31, -2.0**31, 2.0**31 - 1, 2147483647.5,
                           np.nextafter(2.0**31, 0), 5e-324, 2.2250738585072014e-308, 1e-300, 1e-7, 1e-6, 5e-7,
                           np.nan, np.inf, -np.inf, 0.1 + 0.2, 1.0 / 3.0, 123456.789, 2147.483647, 0.000001]))
    v = np.concatenate(parts)
    return v[rng.permutation(len(v))]


def per_value_scales(ops, values, f32=False):
    """cql_fixed_scale in its per-value mode, called through the kernel ABI."""
    from computeql_gb300 import native as N
    lib = N.load_cuda()
    n = len(values)
    src = ops.DeviceBuffer(values.nbytes, values)
    res = ops.DeviceBuffer(16, np.zeros(4, dtype=np.uint32))
    out = ops.DeviceBuffer(max(n, 16))
    k = lib.cqlcuda_kernel_alloc(b"cql_fixed_scale", 15)
    lib.cqlcuda_kernel_set_arg_buffer(k, 0, src.handle)
    lib.cqlcuda_kernel_set_arg_buffer(k, 1, res.handle)
    lib.cqlcuda_kernel_set_arg_buffer(k, 2, res.handle)
    lib.cqlcuda_kernel_set_arg_buffer(k, 3, out.handle)
    lib.cqlcuda_kernel_set_arg_u64(k, 0, n)
    lib.cqlcuda_kernel_set_arg_u64(k, 1, 3 if f32 else 4)
    lib.cqlcuda_kernel_set_arg_u64(k, 2, 0)
    lib.cqlcuda_kernel_set_arg_u64(k, 3, 1)
    got = np.zeros(n, dtype=np.int8)
    b = lib.cqlcuda_batch_begin(0, n)
    lib.cqlcuda_batch_kernel_execute(b, k, n, 256)
    lib.cqlcuda_batch_buffer_read(b, out.handle, C.c_void_p(got.ctypes.data), n)
    assert lib.cqlcuda_batch_end(b), N.last_error()
    return got


def test_per_value_scale_f64(ops):
    v = adversarial_values(400000, 1)
    assert np.array_equal(per_value_scales(ops, v), oracle.fixed_scale_each(v))


def test_per_value_scale_f32(ops):
    v = adversarial_values(200000, 2).astype(np.float32)
    v = v[np.isfinite(v) | np.isnan(v)]
    assert np.array_equal(per_value_scales(ops, v, f32=True), oracle.fixed_scale_each(v.astype(np.float64)))


@pytest.mark.parametrize("places", [0, 1, 2, 3, 4, 6])
def test_column_scale(ops, places):
    rng = np.random.default_rng(places)
    v = rng.integers(-10**8, 10**8, 300000) / 10.0**places
    v[rng.integers(0, len(v), 5)] = 0.5           # a coarser value does not lower the scale
    want = oracle.fixed_scale(v)
    got = ops.fixed_scale(ops.Column.from_numpy(v))
    assert got[0] == want[0] and got[1] == want[1]


def test_column_scale_fails_like_the_reference(ops):
    rng = np.random.default_rng(5)
    cases = [rng.normal(size=1000), np.array([1.5, 2.0**31]), np.array([0.1234567]), np.array([3000.5, 1.0e-6]),
             np.array([2147.483647, 1.0]), np.array([np.nan])]
    for v in cases:
        got = ops.fixed_scale(ops.Column.from_numpy(v))[0]
        assert got == oracle.fixed_scale(v)[0]


def _check_group(ops, key, funcs, args, selection=None):
    rows = None if selection is None else np.asarray(selection)
    kcol = ops.Column.from_numpy(key)
    acols = [ops.Column.from_numpy(a) if a is not None else None for a in args]
    sel = ops.DeviceBuffer(rows.nbytes, rows.astype(np.uint32)) if rows is not None else None
    got = ops.group_dense_fixed(kcol, funcs, acols, selection=sel)
    pick = (lambda x: x) if rows is None else (lambda x: x[rows])
    scales = [0 if f == COUNT else oracle.fixed_scale(pick(a).astype(np.float64))[0] for f, a in zip(funcs, args)]
    assert got["scales"] == scales
    want = oracle.dense_fixed(pick(key).astype(np.float64), funcs,
                              [pick(a).astype(np.float64) if a is not None else None for a in args], scales)
    assert np.array_equal(got["keys"], want["keys"])
    assert np.array_equal(got["counts"], want["counts"])
    first = want["first_rows"] if rows is None else rows[want["first_rows"].astype(np.int64)]
    assert np.array_equal(got["first_rows"], first)
    assert np.array_equal(got["results"].view(np.uint64), want["results"].view(np.uint64))   # bit for bit


@pytest.mark.parametrize("key_dtype", [np.uint32, np.int32, np.float64])
def test_group_by_prices(ops, key_dtype):
    rng = np.random.default_rng(8)
    n = 2_000_000
    key = rng.integers(0, 50, n).astype(key_dtype) if key_dtype != np.int32 else rng.integers(-25, 25, n).astype(np.int32)
    price = rng.integers(-500000, 500000, n) / 100.0
    qty = rng.integers(0, 1000, n) / 1000.0
    _check_group(ops, key, [COUNT, SUM, AVG, MIN, MAX, SUM], [None, price, price, price, price, qty])


def test_group_by_f32_arguments(ops):
    rng = np.random.default_rng(9)
    n = 1_000_000
    key = rng.integers(0, 5, n).astype(np.uint32)
    amount = (rng.integers(0, 100000, n) / 4.0).astype(np.float32)       # quarters: exact in f32
    _check_group(ops, key, [SUM, MIN, MAX, AVG], [amount, amount, amount, amount])


def test_group_by_large_sums_and_scale_6(ops):
    rng = np.random.default_rng(10)
    n = 4_000_000
    key = rng.integers(0, 3, n).astype(np.uint32)
    v = rng.integers(-2**31 + 1, 2**31, n) / 1e6       # the doubles nearest 6-place decimals, |v * 10^6| < 2^31
    _check_group(ops, key, [SUM, AVG, MIN, MAX], [v, v, v, v])


def test_group_by_selection(ops):
    rng = np.random.default_rng(11)
    n = 3_000_000
    key = rng.integers(100, 300, n).astype(np.int32)
    price = rng.integers(0, 10**6, n) / 1000.0
    rows = np.nonzero(rng.random(n) < 0.07)[0]
    _check_group(ops, key, [COUNT, SUM, MAX], [None, price, price], selection=rows)


def test_refuses_non_decimals(ops):
    key = np.zeros(1000, dtype=np.uint32)
    v = np.random.default_rng(1).normal(size=1000)
    from computeql_gb300.ops import OpError
    with pytest.raises(OpError, match="decimal"):
        ops.group_dense_fixed(ops.Column.from_numpy(key), [SUM], [ops.Column.from_numpy(v)])


def test_reference_kernel_contract(ops):
    """aggregate_dense_f64 with the reference's bindings: f64 keys, f64 arguments, host-side scales."""
    from computeql_gb300 import native as N
    lib = N.load_cuda()
    rng = np.random.default_rng(12)
    n, G = 500000, 40
    keys = rng.integers(7, 7 + G, n).astype(np.float64)
    a0 = rng.integers(-10**6, 10**6, n) / 100.0
    funcs = [COUNT, SUM, MIN, MAX]
    scales = [0, 2, 2, 2]
    bufs = {"k": ops.DeviceBuffer(keys.nbytes, keys), "a": ops.DeviceBuffer(a0.nbytes, a0),
            "info": ops.DeviceBuffer(G * 8, np.zeros(G * 2, dtype=np.uint32)),
            "sum": ops.DeviceBuffer(G * 4 * 8, np.zeros(G * 4, dtype=np.int64)),
            "min": ops.DeviceBuffer(G * 4 * 4, np.full(G * 4, 0x7fffffff, dtype=np.int32)),
            "max": ops.DeviceBuffer(G * 4 * 4, np.full(G * 4, -0x80000000, dtype=np.int32))}
    k = lib.cqlcuda_kernel_alloc(b"aggregate_dense_f64", 19)
    for i, name in enumerate(["k", "info", "sum", "min", "max"]):
        lib.cqlcuda_kernel_set_arg_buffer(k, i, bufs[name].handle)
    for e in range(8):
        lib.cqlcuda_kernel_set_arg_buffer(k, 5 + e, bufs["a"].handle)
    codes = sum(f << (4 * e) for e, f in enumerate(funcs))
    sc = sum(s << (4 * e) for e, s in enumerate(scales))
    for slot, v in enumerate([n, len(funcs), codes, sc, G, 7]):
        lib.cqlcuda_kernel_set_arg_u64(k, slot, v)
    lib.cqlcuda_kernel_execute(k, (n + 16383) // 16384 * 256, 256)
    lib.cqlcuda_wait()
    info = bufs["info"].read(np.uint32).reshape(G, 2)
    sums = bufs["sum"].read(np.int64).reshape(G, 4)
    mins = bufs["min"].read(np.int32).reshape(G, 4)
    maxs = bufs["max"].read(np.int32).reshape(G, 4)
    want = oracle.dense_fixed(keys, funcs, [None, a0, a0, a0], scales)
    assert np.array_equal(info[:, 1], want["counts"])
    assert np.array_equal(~info[:, 0], want["first_rows"].astype(np.uint32))
    assert np.array_equal(sums[:, 1] / 100.0, want["results"][:, 1])
    assert np.array_equal(mins[:, 2] / 100.0, want["results"][:, 2])
    assert np.array_equal(maxs[:, 3] / 100.0, want["results"][:, 3])


def test_reference_resident_table(ops):
    """SELECT grp, SUM(dv), MIN(dv), MAX(dv) FROM t GROUP BY grp on the table of bench_query_agg_resident.c."""
    from tests.test_fixed_oracle import ar_table
    grp, wv, cents, dv = ar_table()
    _check_group(ops, grp, [SUM, MIN, MAX], [dv, dv, dv])
    # the filtered form (:207): SELECT grp, SUM(dv) FROM t WHERE wv > 500 GROUP BY grp
    _check_group(ops, grp, [SUM], [dv], selection=np.nonzero(wv > 500)[0])
