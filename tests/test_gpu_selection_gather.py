"""The reference-named selection_gather kernel through the backend ABI, every row-map mode (GB300 only).

qe_selection_gather_column (src/query_exec/query_exec.c:4371) and qe_rows_resolve (:4476) dispatch
`selection_gather` by name with the bindings and push words of selection_gather.comp:17-35: binding 0 the
rows (one index every `stride` words, at `word_offset`), 1 the source, 2 the destination, 3 positions;
words 0 count, 2 stride, 4 row offset, 6 mode, 8 map stride, 10 word offset, 12 map offset. Each mode is
compared word for word with the oracle's restatement of :28-78, including rows that are 0xffffffff (no
row), strided row lists such as a join's (probe, build) pairs, and offsets.
"""
import ctypes as C

import numpy as np
import pytest

import oracle

pytestmark = pytest.mark.gpu
NO_ROW = 0xFFFFFFFF


@pytest.fixture(scope="module")
def lib(gpu):
    return gpu.load_cuda()


def buf(lib, arr):
    arr = np.ascontiguousarray(arr, dtype=np.uint32)
    h = lib.cqlcuda_buffer_alloc(max(arr.nbytes, 4), 0, C.c_void_p(arr.ctypes.data) if arr.nbytes else None)
    assert h, lib.cqlcuda_last_error()
    return h


def run(lib, mode, rows, source, positions, count, stride=1, row_offset=0, map_stride=1, word_offset=0, map_offset=0):
    k = lib.cqlcuda_kernel_alloc(b"selection_gather", 16)
    assert k
    out_words = count * (2 if mode == 0 else 1)
    handles = [buf(lib, rows), buf(lib, source if source is not None else np.zeros(1, np.uint32)),
               buf(lib, np.full(max(out_words, 1), 0xDEADBEEF, dtype=np.uint32)),
               buf(lib, positions if positions is not None else np.zeros(1, np.uint32))]
    for i, h in enumerate(handles):
        lib.cqlcuda_kernel_set_arg_buffer(k, i, h)
    for slot, v in enumerate((count, stride, row_offset, mode, map_stride, word_offset, map_offset)):
        lib.cqlcuda_kernel_set_arg_u64(k, slot, v)
    out = np.zeros(max(out_words, 1), dtype=np.uint32)
    b = lib.cqlcuda_batch_begin(0, out.nbytes)
    lib.cqlcuda_batch_kernel_execute(b, k, max(count, 1), 256)
    lib.cqlcuda_batch_buffer_read(b, handles[2], C.c_void_p(out.ctypes.data), out.nbytes)
    assert lib.cqlcuda_batch_end(b) == 1, lib.cqlcuda_last_error()
    for h in handles:
        lib.cqlcuda_buffer_release(h)
    return out[:out_words]


def with_holes(rng, n, hi, frac=0.1):
    r = rng.integers(0, hi, n).astype(np.uint32)
    r[rng.random(n) < frac] = NO_ROW
    return r


@pytest.mark.parametrize("count", [1, 1000, 300_001])
def test_f64_and_u32_columns_through_rows(lib, count):
    rng = np.random.default_rng(count)
    src64 = rng.normal(0, 1e6, 50_000).view(np.uint32)          # f64 values as word pairs
    src32 = rng.integers(0, 1 << 32, 50_000, dtype=np.uint64).astype(np.uint32)
    rows = with_holes(rng, count, 49_000)
    for mode, src in ((0, src64), (1, src32)):
        got = run(lib, mode, rows, src, None, count, row_offset=7)
        want = oracle.selection_gather(mode, rows, src, None, count, row_offset=7)
        assert np.array_equal(got, want), mode


def test_strided_pairs_pick_one_side(lib):
    """A join's (probe, build) pairs: stride 2, word offset 1 reads the build rows; unmatched LEFT rows
    (0xffffffff) read as 0."""
    rng = np.random.default_rng(5)
    n = 20_000
    pairs = np.stack([np.arange(n, dtype=np.uint32), with_holes(rng, n, 9_000, 0.2)], axis=1).ravel()
    src = rng.integers(0, 1 << 31, n).astype(np.uint32)          # probe rows reach n - 1
    for word_offset in (0, 1):
        got = run(lib, 1, pairs, src, None, n, stride=2, word_offset=word_offset)
        assert np.array_equal(got, oracle.selection_gather(1, pairs, src, None, n, stride=2, word_offset=word_offset))


def test_positions_mode(lib):
    rng = np.random.default_rng(6)
    rows = with_holes(rng, 40_000, 1_000_000)
    positions = rng.integers(0, 20_000, 15_000).astype(np.uint32)
    got = run(lib, 2, rows, None, positions, len(positions), stride=2, row_offset=1000, word_offset=1)
    want = oracle.selection_gather(2, rows, None, positions, len(positions), stride=2, row_offset=1000, word_offset=1)
    assert np.array_equal(got, want)


def test_resolve_modes(lib):
    rng = np.random.default_rng(7)
    rows = with_holes(rng, 30_000, 5_000)
    mapping = with_holes(rng, 3 * 5_000, 2_000_000)          # a map read every 3 words
    got = run(lib, 3, rows, mapping, None, len(rows), map_stride=3, map_offset=11)
    assert np.array_equal(got, oracle.selection_gather(3, rows, mapping, None, len(rows), map_stride=3, map_offset=11))
    got = run(lib, 4, rows, None, None, len(rows), row_offset=123)
    assert np.array_equal(got, oracle.selection_gather(4, rows, None, None, len(rows), row_offset=123))


def test_zero_count_writes_nothing(lib):
    rows = np.array([1, 2, 3], dtype=np.uint32)
    assert len(run(lib, 1, rows, np.arange(10, dtype=np.uint32), None, 0)) == 0
