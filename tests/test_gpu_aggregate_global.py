"""aggregate_global_native through the C ABI against the oracle and the reference's known answers.

Whole-number columns must match bit for bit; F64/F32 sums within 1e-12 relative of the reference
GPU order (the oracle's restatement of it), and the error against a compensated sum is reported.
"""
import json
import os

import numpy as np
import pytest

import oracle
from tests import closed_form as cf

pytestmark = pytest.mark.gpu
GOLDEN = os.path.join(os.path.dirname(__file__), "golden")
F64_RTOL = 1e-12


@pytest.fixture(scope="module")
def ops(gpu):
    from computeql_gb300 import ops as o
    return o


def test_c1_sum_min_max_amount_matches_golden(ops):
    from computeql_gb300 import workloads
    fx = json.load(open(os.path.join(GOLDEN, "c1_oracle.json")))
    t = workloads.fact_table(fx["rows"])
    s, mn, mx = ops.aggregate_global([t.amount])
    assert [s[0], mn[0], mx[0]] == fx["sum_min_max_amount"]
    assert ops.launches() >= 1


def test_device_generator_matches_oracle_generator(ops):
    from computeql_gb300 import workloads
    n = 1_000_003
    t = workloads.fact_table(n)
    h = workloads.fact_numpy(n, gen=oracle.splitmix_u32)
    for name in ("region", "amount", "flag"):
        got = getattr(t, name).buffer.read(np.uint32, n)
        assert np.array_equal(got, h[name]), name


@pytest.mark.parametrize("n", [1, 2, 3, 4, 5, 7, 16, 17, 1000, 10001, 1000003, 10_000_000])
def test_closed_form_sum_min_max(ops, n):
    _, _, amount, _ = oracle.closed_form(n)
    col = ops.Column.from_numpy(amount)
    s, mn, mx = ops.aggregate_global([col])
    assert [s[0], mn[0], mx[0]] == cf.expected(n)["sum_min_max_amount"]


@pytest.mark.parametrize("n", [0, 1, 3, 5, 64, 1023, 99991, 2_000_001])
@pytest.mark.parametrize("dtype", [np.uint32, np.int32])
def test_whole_number_columns_bit_exact(ops, n, dtype):
    rng = np.random.default_rng(n + 7)
    if dtype == np.uint32:
        a = rng.integers(0, 2**32, n, dtype=np.uint64).astype(np.uint32)
    else:
        a = rng.integers(-2**31, 2**31, n, dtype=np.int64).astype(np.int32)
    s, mn, mx = ops.aggregate_global([ops.Column.from_numpy(a)])
    es, emn, emx = oracle.aggregate_global_gpu_order(a)
    exact = float(a.astype(np.int64).sum()) if n else 0.0
    assert s[0] == exact
    assert (mn[0], mx[0]) == (emn, emx)
    if abs(exact) < 2**53:
        assert s[0] == es


@pytest.mark.parametrize("n", [1, 2, 3, 5, 77, 4096, 100003, 3_000_001])
@pytest.mark.parametrize("dtype", [np.float32, np.float64])
def test_float_columns_within_tolerance(ops, n, dtype):
    rng = np.random.default_rng(n)
    a = (rng.lognormal(3.0, 1.0, n) * rng.choice([-1.0, 1.0], n)).astype(dtype)
    s, mn, mx = ops.aggregate_global([ops.Column.from_numpy(a)])
    ref_s, ref_mn, ref_mx = oracle.aggregate_global_gpu_order(a)
    comp = oracle.compensated_sum(a)
    assert (mn[0], mx[0]) == (ref_mn, ref_mx)
    scale = max(abs(ref_s), float(np.abs(a.astype(np.float64)).sum()) * 1e-3, 1e-300)
    assert abs(s[0] - ref_s) <= F64_RTOL * scale
    assert abs(s[0] - comp) <= F64_RTOL * scale


@pytest.mark.parametrize("width,span", [(1, 200), (2, 60000)])
@pytest.mark.parametrize("n", [1, 15, 16, 17, 1000, 1_048_579])
def test_narrow_columns(ops, width, span, n):
    rng = np.random.default_rng(width * 1000 + n)
    base = 123456
    a = (base + rng.integers(0, span, n)).astype(np.uint32)
    col = ops.Column.from_numpy(a, narrow=True)
    assert col.width == (1 if a.max() - a.min() < 256 else 2)
    s, mn, mx = ops.aggregate_global([col])
    assert s[0] == float(a.astype(np.int64).sum())
    assert (mn[0], mx[0]) == (float(a.min()), float(a.max()))


def test_narrow_signed_column(ops):
    rng = np.random.default_rng(3)
    a = rng.integers(-1000, -800, 100001).astype(np.int32)
    col = ops.Column.from_numpy(a, narrow=True)
    assert col.width == 1
    s, mn, mx = ops.aggregate_global([col])
    assert (s[0], mn[0], mx[0]) == (float(a.astype(np.int64).sum()), float(a.min()), float(a.max()))


def test_sequence_column_closed_form(ops):
    n = 1_000_000
    s, mn, mx = ops.aggregate_global([ops.Column.sequence(n, 1)])
    assert (s[0], mn[0], mx[0]) == (float(n * (n + 1) // 2), 1.0, float(n))
    assert ops.launches() == 0


def test_four_columns_in_one_launch(ops):
    rng = np.random.default_rng(11)
    n = 500_001
    cols = [rng.integers(0, 1000, n).astype(np.uint32), rng.integers(-5, 5, n).astype(np.int32),
            rng.random(n).astype(np.float64), rng.random(n).astype(np.float32)]
    s, mn, mx = ops.aggregate_global([ops.Column.from_numpy(c) for c in cols])
    for i, c in enumerate(cols):
        es, emn, emx = oracle.aggregate_global_gpu_order(c)
        assert (mn[i], mx[i]) == (emn, emx)
        assert abs(s[i] - es) <= F64_RTOL * max(abs(es), 1.0)
    assert ops.launches() == 1
