"""Zone-map pruning of scans (cqlops_scan_ranges), host logic only: runs without a GPU.

The rules are qe_scan_build_dispatch_ranges (src/query_exec/query_exec.c:13307-13540) for a table in
one buffer: a chunk of 8192 rows goes when a leaf proves it empty (qe_zonemap_chunk_is_prunable,
:13294-13304); an interior gap under 1M rows is scanned anyway; nothing goes unless 10% of the rows
do; kept chunks merge into ranges, or one pass with a skip bitmap when the ranges cost more.
"""
import ctypes as C

import numpy as np
import pytest

CHUNK = 8192
EQ, LT, LE, GT, GE = 0, 1, 2, 3, 4


@pytest.fixture(scope="module")
def N():
    from computeql_gb300 import build, native
    build.build()
    native.load_ops()
    return native


def col(N, rows, ctype=1, width=0, base=0, zone_map=None, keep=None):
    c = N.CqlColumn()
    c.type, c.width, c.base, c.rows = ctype, width, base, rows
    c.buffer = None if width == 3 else 1   # never dereferenced on the host
    if zone_map is not None:
        pairs = zone_map.reshape(-1, 2)
        has = pairs[:, 0] <= pairs[:, 1]
        summary = [pairs[has, 0].max(), pairs[has, 1].min()] if has.any() else [-np.inf, np.inf]
        zone_map = np.concatenate([zone_map, summary])      # the chunks, then (largest min, smallest max)
        keep.append(zone_map)
        c.zone_map = zone_map.ctypes.data
        c.zone_map_chunks = len(zone_map) // 2 - 1
    return c


def ranges(N, cols, leaves, max_ranges=64):
    arr = (N.CqlColumn * len(cols))(*cols)
    lv = (N.CqlLeaf * len(leaves))(*[N.CqlLeaf(c, op, t) for c, op, t in leaves])
    rows = cols[0].rows
    chunks = (rows + CHUNK - 1) // CHUNK
    out = np.zeros(2 * max_ranges, dtype=np.uint64)
    skip = np.zeros((chunks + 31) // 32 + 1, dtype=np.uint32)
    use_skip = C.c_int()
    pruned = C.c_uint64()
    n = N.load_ops().cqlops_scan_ranges(arr, len(cols), lv, len(leaves), out.ctypes.data, max_ranges, skip.ctypes.data,
                                        C.byref(use_skip), C.byref(pruned))
    return [tuple(int(x) for x in out[2 * i:2 * i + 2]) for i in range(min(n, max_ranges))], use_skip.value, pruned.value, skip


def test_point_lookup_on_a_sequence_keeps_one_chunk(N):
    rows = 1_000_000_000
    k = 123_456_789
    r, skip, pruned, _ = ranges(N, [col(N, rows, width=3)], [(0, EQ, k)])
    start = k // CHUNK * CHUNK
    assert r == [(start, start + CHUNK)] and not skip and pruned == rows - CHUNK


def test_range_predicate_on_a_sequence(N):
    rows = 100_000_000
    r, skip, pruned, _ = ranges(N, [col(N, rows, width=3, base=1000)], [(0, LT, 5_001_000)])
    assert r == [(0, 5_005_312)] and pruned == rows - 5_005_312
    # a non-whole target and >=
    r, _, _, _ = ranges(N, [col(N, rows, width=3)], [(0, GE, 99_000_000.5)])
    assert r == [((99_000_001 // CHUNK) * CHUNK, rows)]


def test_less_than_ten_percent_is_not_pruned(N):
    rows = 10_000_000
    r, skip, pruned, _ = ranges(N, [col(N, rows, width=3)], [(0, GE, 500_000)])
    assert r == [(0, rows)] and pruned == 0


def test_no_usable_leaf_scans_everything(N):
    rows = 50_000_000
    r, skip, pruned, _ = ranges(N, [col(N, rows)], [(0, LT, 2)])     # no zone map
    assert r == [(0, rows)] and pruned == 0


def test_zone_map_and_short_gaps(N):
    keep = []
    rows = 64 * CHUNK * 100
    chunks = rows // CHUNK
    zm = np.zeros(2 * chunks)
    zm[0::2] = 0.0
    zm[1::2] = 10.0
    hot = [5, 6, 7, 200, 4000, 6000]
    for z in hot:
        zm[2 * z + 1] = 100.0          # only these chunks can hold values > 50
    c = col(N, rows, zone_map=zm, keep=keep)
    r, skip, pruned, bits = ranges(N, [c], [(0, GT, 50.0)])
    # the gap 8..199 (192 chunks) is at least 1M rows (128 chunks): pruned; 201..3999 too; kept: 5-7, 200, 4000, 6000
    assert not skip
    assert r == [(5 * CHUNK, 8 * CHUNK), (200 * CHUNK, 201 * CHUNK), (4000 * CHUNK, 4001 * CHUNK), (6000 * CHUNK, 6001 * CHUNK)]
    # a gap shorter than 128 chunks between kept chunks is scanned
    zm2 = zm.copy()
    zm2[2 * 100 + 1] = 100.0           # gaps 8..99 and 101..199 are under 128 chunks: scanned
    c2 = col(N, rows, zone_map=zm2, keep=keep)
    r2, _, _, _ = ranges(N, [c2], [(0, GT, 50.0)])
    assert r2[:2] == [(5 * CHUNK, 201 * CHUNK), (4000 * CHUNK, 4001 * CHUNK)]


def test_many_ranges_become_a_skip_bitmap(N):
    keep = []
    rows = 20_000_000
    chunks = (rows + CHUNK - 1) // CHUNK
    zm = np.zeros(2 * chunks)
    zm[1::2] = 1.0
    kept = list(range(0, chunks, 200))   # kept chunks every 200: many ranges, each a cost of 4M rows
    for z in kept:
        zm[2 * z + 1] = 9.0
    c = col(N, rows, zone_map=zm, keep=keep)
    r, skip, pruned, bits = ranges(N, [c], [(0, GE, 5.0)])
    assert skip == 1 and r == [(0, rows)]
    for z in range(chunks):
        assert bool(bits[z >> 5] & (1 << (z & 31))) == (z not in kept)


def test_summary_short_cuts_a_leaf_that_prunes_nothing(N):
    keep = []
    rows = 1_000_000
    chunks = (rows + CHUNK - 1) // CHUNK
    zm = np.tile([0.0, 99.0], chunks)
    r, skip, pruned, _ = ranges(N, [col(N, rows, zone_map=zm, keep=keep)], [(0, LT, 2.0)])
    assert r == [(0, rows)] and pruned == 0


def test_everything_pruned(N):
    keep = []
    rows = 1_000_000
    chunks = (rows + CHUNK - 1) // CHUNK
    zm = np.tile([0.0, 1.0], chunks)
    r, skip, pruned, _ = ranges(N, [col(N, rows, zone_map=zm, keep=keep)], [(0, EQ, 7.0)])
    assert r == [] and pruned == rows
