"""The resident chunk cache over device buffers (the default allocator): a query streams a host column
through it chunk by chunk, the second pass finds every chunk resident, and the kernels read the cached
buffers as columns."""
import ctypes as C

import numpy as np
import pytest

pytestmark = pytest.mark.gpu


class Handle:
    def __init__(self, h):
        self.handle = h


def test_chunks_are_kept_between_queries(gpu):
    from computeql_gb300 import native, ops
    lib = native.load_ops()
    cache = lib.cqlops_resident_create(0, None)
    assert cache
    rng = np.random.default_rng(2)
    n, chunk = 4_000_000, 1 << 20
    host = rng.integers(0, 1 << 20, n).astype(np.uint32)
    want = float(host.astype(np.float64).sum())
    for query in range(2):
        total, hits = 0.0, 0
        for first in range(0, n, chunk):
            rows = min(chunk, n - first)
            hit = C.c_int()
            buf = lib.cqlops_resident_acquire(cache, 77, 1, host[first:].ctypes.data, first, rows, 4, C.byref(hit))
            assert buf
            hits += hit.value
            col = ops.Column(ops.TYPE_U32, rows, Handle(buf), zone=(0.0, float((1 << 20) - 1)), zone_map=False)
            total += ops.aggregate_global([col])[0][0]
            lib.cqlops_resident_release(cache, buf)
        assert total == want
        assert hits == (0 if query == 0 else 4)
    st = lib.cqlops_resident_stats(cache)
    assert st.entries == 4 and st.bytes_in_use == n * 4 and st.hit_bytes == n * 4 and st.miss_bytes == n * 4
    assert st.budget_bytes > n * 4
    # a write to the column (a new generation) is never served from the old copy
    host2 = host + 1
    hit = C.c_int()
    buf = lib.cqlops_resident_acquire(cache, 77, 2, host2.ctypes.data, 0, chunk, 4, C.byref(hit))
    assert buf and not hit.value
    out = np.empty(chunk, dtype=np.uint32)
    native.load_cuda().cqlcuda_buffer_read(buf, out.ctypes.data, chunk * 4)
    assert np.array_equal(out, host2[:chunk])
    lib.cqlops_resident_release(cache, buf)
    lib.cqlops_resident_destroy(cache)


@pytest.mark.parametrize("dtype", [np.uint32, np.int32, np.float64])
def test_streamed_aggregate_over_the_cache(gpu, dtype):
    """SUM/MIN/MAX of a host column streamed through the cache: the first pass uploads every chunk, the
    second uploads nothing and gives the same answer; a written column (a new generation) is uploaded again.
    Integer sums exact; f64 within 1e-12 of a compensated sum."""
    import oracle
    from computeql_gb300 import native, ops
    lib = native.load_ops()
    cache = lib.cqlops_resident_create(0, None)
    rng = np.random.default_rng(3)
    n, chunk = 3_000_001, 1 << 20
    if dtype == np.float64:
        host = rng.lognormal(3.0, 1.0, n)
    else:
        host = rng.integers(-2**30 if dtype == np.int32 else 0, 2**30, n).astype(dtype)
    ctype = {np.uint32: ops.TYPE_U32, np.int32: ops.TYPE_I32, np.float64: ops.TYPE_F64}[dtype]
    width = host.itemsize
    results = []
    for generation in (1, 1, 2):
        s, mn, mx, up = C.c_double(), C.c_double(), C.c_double(), C.c_uint64()
        assert lib.cqlops_aggregate_global_streamed(cache, 9, generation, host.ctypes.data, ctype, n, chunk, C.byref(s), C.byref(mn),
                                                    C.byref(mx), C.byref(up)), native.last_error()
        results.append((s.value, mn.value, mx.value, up.value))
    assert [r[3] for r in results] == [n * width, 0, n * width]
    assert results[0][:3] == results[1][:3] == results[2][:3]
    s, mn, mx, _ = results[0]
    assert (mn, mx) == (float(host.min()), float(host.max()))
    if dtype == np.float64:
        exact = oracle.compensated_sum(host)
        assert abs(s - exact) <= 1e-12 * abs(exact)
    else:
        assert s == float(host.astype(np.int64).sum())
    lib.cqlops_resident_destroy(cache)
