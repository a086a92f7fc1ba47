"""HAVING over grouped results on the GPU (cqlops_having, the reference's qk_having_kernel contract):
each group's flag equals the condition evaluated in double on the host; conditions differing only in
literals share a kernel; conditions with anything but v0..v7, lit[i], numbers, operators and the listed
functions are refused before any compile."""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def ops(gpu):
    from computeql_gb300 import ops as o
    return o


def test_conditions_match_the_host(ops):
    rng = np.random.default_rng(9)
    g = 70_001
    count = rng.integers(0, 1000, g).astype(np.float64)
    total = rng.normal(0.0, 1000.0, g)
    avg = total / np.maximum(count, 1.0)
    cases = [
        ("v0 > lit[0]", [count], [500.0], lambda: count > 500.0),
        ("v0 >= lit[0] && v1 < lit[1]", [count, total], [100.0, 0.0], lambda: (count >= 100.0) & (total < 0.0)),
        ("!(v0 == lit[0]) || fabs(v1) > lit[1]", [count, total], [7.0, 2500.0], lambda: (count != 7.0) | (np.abs(total) > 2500.0)),
        ("v2 * 2.0 - v1 / 4.0 > lit[0]", [count, total, avg], [-3.5], lambda: avg * 2.0 - total / 4.0 > -3.5),
        ("fmax(v0, v1) <= lit[0] && !isnan(v2)", [count, total, avg], [600.0], lambda: np.maximum(count, total) <= 600.0),
    ]
    for cond, cols, lits, want in cases:
        keep = ops.having(cond, cols, lits)
        assert np.array_equal(keep.astype(bool), want()), cond


def test_literals_share_one_kernel(ops):
    from computeql_gb300 import native
    import ctypes as C
    lib = native.load_cuda()
    v = np.arange(1000, dtype=np.float64)
    ops.having("v0 < lit[0]", [v], [10.0])
    compiles = C.c_uint64()
    lib.cqlcuda_generated_kernel_stats(C.byref(compiles), None)
    before = compiles.value
    for t in (20.0, 300.0, 999.5):
        assert ops.having("v0 < lit[0]", [v], [t]).sum() == int(np.ceil(t))
    lib.cqlcuda_generated_kernel_stats(C.byref(compiles), None)
    assert compiles.value == before


@pytest.mark.parametrize("cond", ["v0 > 1; keep[0] = 2", "printf(0)", "v9 > 1", "v0 > 1 } {", '"x"', "#define X"])
def test_other_text_is_refused(ops, cond):
    with pytest.raises(ops.OpError):
        ops.having(cond, [np.zeros(4)], [])
