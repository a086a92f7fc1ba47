"""The generated-kernel cap: past it the least recently used NVRTC kernel is unloaded and counted, and a
shape whose kernel was evicted compiles again and still answers right (GB300 only).

The reference caps its generated pipelines at GPU_VULKAN_MAX_GENERATED_KERNELS (default 64, at least 8)
and evicts the least recently used (src/gpu/vulkan/gpu_vulkan.c:75, :2721-2737), counting evictions in
generated_kernel_stats; a long-running server meeting new WHERE shapes would otherwise keep every module
loaded.
"""
import ctypes as C

import numpy as np
import pytest

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def env(gpu):
    from computeql_gb300 import ops
    rng = np.random.default_rng(21)
    flag = rng.integers(0, 100, 300_000).astype(np.uint32)
    amount = rng.integers(0, 10_000, 300_000).astype(np.uint32)
    cols = {"flag": ops.Column.from_numpy(flag), "amount": ops.Column.from_numpy(amount)}
    lib = gpu.load_cuda()
    yield ops, lib, cols, flag, amount
    lib.cqlcuda_set_generated_kernel_cap(64)


def stats(lib):
    c, e = C.c_uint64(), C.c_uint64()
    lib.cqlcuda_generated_kernel_stats(C.byref(c), C.byref(e))
    return c.value, e.value


def shape(k):
    """a distinct WHERE shape per k: an OR chain of k equalities, AND a range on amount"""
    terms = [f"(= flag {3 * j})" for j in range(k)]
    chain = terms[0]
    for t in terms[1:]:
        chain = f"(or {chain} {t})"
    return f"(and {chain} (< amount {5000 + k}))"


def expected(k, flag, amount):
    hit = np.zeros(len(flag), dtype=bool)
    for j in range(k):
        hit |= flag == 3 * j
    return int((hit & (amount < 5000 + k)).sum())


def test_cap_evicts_least_recently_used_and_recompiles(env):
    ops, lib, cols, flag, amount = env
    lib.cqlcuda_set_generated_kernel_cap(8)
    c0, e0 = stats(lib)
    shapes = 20
    for k in range(1, shapes + 1):
        count, _, _ = ops.scan_filter(ops.Program(shape(k), cols), strategy=ops.SCAN_GENERATED)
        assert count == expected(k, flag, amount), k
    c1, e1 = stats(lib)
    assert c1 - c0 >= shapes                   # every shape was new
    assert e1 - e0 >= shapes - 8               # at most 8 generated kernels stay loaded
    # the first shape was evicted: it compiles again and answers right
    count, _, _ = ops.scan_filter(ops.Program(shape(1), cols), strategy=ops.SCAN_GENERATED)
    assert count == expected(1, flag, amount)
    c2, e2 = stats(lib)
    assert c2 == c1 + 1 and e2 >= e1 + 1
    # a recent shape is still loaded: no compile
    count, _, _ = ops.scan_filter(ops.Program(shape(shapes), cols), strategy=ops.SCAN_GENERATED)
    assert count == expected(shapes, flag, amount)
    assert stats(lib)[0] == c2
