"""Row counts past the kernels' 32-bit row numbers are refused, not truncated (CPU only).

Every kernel takes its row count and row numbers as 32-bit push-constant words, as the reference's
shaders do (the reference never passes more than a 16M-row chunk, query_exec.c:2097). A column
descriptor of 5 x 10^9 rows (20 GB of u32, which one GB300 holds) with no device buffer behind it
must make every operator return 0 with a message, before any allocation or launch: the descriptor
has no buffer, so a call that went on would fault on the host or read nothing.
"""
import ctypes as C

import numpy as np
import pytest

from computeql_gb300 import native as N
from computeql_gb300 import ops

BIG = 5_000_000_000


@pytest.fixture(scope="module")
def lib():
    from computeql_gb300 import build
    build.build()
    return N.load_ops()


def big(ctype=ops.TYPE_U32, zone=(0.0, 49.0)):
    col = N.CqlColumn()
    col.type = ctype
    col.rows = BIG
    col.has_range = 1
    col.zone_min, col.zone_max = zone
    return col


def refused(lib, rc):
    assert rc == 0
    msg = lib.cqlops_last_error().decode()
    assert "5000000000 rows" in msg and "at most 4294967294 rows" in msg, msg


def test_max_rows_constant_matches_the_header():
    text = open(__import__("os").path.join(ops.__file__.rsplit("/", 2)[0], "include", "cqlops.h")).read()
    assert "#define CQLOPS_MAX_ROWS 0xfffffffeull" in text


def test_aggregate_global_refuses(lib):
    cols = (N.CqlColumn * 1)(big())
    s, mn, mx = (C.c_double * 1)(), (C.c_double * 1)(), (C.c_double * 1)()
    refused(lib, lib.cqlops_aggregate_global(cols, 1, s, mn, mx))


def test_scan_simple_refuses(lib):
    cols = (N.CqlColumn * 1)(big())
    leaves = (N.CqlLeaf * 1)(N.CqlLeaf(0, ops.CMP_LT, 2.0))
    cnt = C.c_uint64()
    refused(lib, lib.cqlops_scan_simple(cols, 1, leaves, 1, C.byref(cnt), None, 0))


def test_group_dense_refuses(lib):
    key = big()
    funcs = np.array([ops.FUNC_COUNT], dtype=np.uint32)
    args = (C.c_void_p * 1)(None)
    g, mk = C.c_uint64(), C.c_int64()
    out = np.zeros(64, dtype=np.int64)
    refused(lib, lib.cqlops_group_dense(C.byref(key), BIG, 1, N.ptr(funcs), args, 64, C.byref(g), C.byref(mk), N.ptr(out), N.ptr(out),
                                        N.ptr(out), N.ptr(out)))


def test_group_hash_refuses(lib):
    keys = (N.CqlColumn * 1)(big())
    funcs = np.array([ops.FUNC_COUNT], dtype=np.uint32)
    args = (C.c_void_p * 1)(None)
    g, used = C.c_uint64(), C.c_uint32()
    out = np.zeros(8, dtype=np.float64)
    refused(lib, lib.cqlops_group_hash(keys, 1, 1, N.ptr(funcs), args, None, 0, 1, 8, C.byref(g), N.ptr(out), N.ptr(out), N.ptr(out),
                                       C.byref(used)))


def test_scan_filter_refuses(lib):
    cols = {"flag": ops.Column(ops.TYPE_U32, BIG, zone=(0.0, 99.0))}
    prog = ops.Program("(< flag 2)", cols)
    arr = (N.CqlColumn * 1)(big(zone=(0.0, 99.0)))
    cnt, used = C.c_uint64(), C.c_uint32()
    refused(lib, lib.cqlops_scan_filter(C.byref(prog.prog), arr, 0, C.byref(cnt), None, 0, C.byref(used)))
    s = (C.c_double * 1)()
    aggs = np.array([0], dtype=np.uint32)
    refused(lib, lib.cqlops_fused_filter_aggregate(C.byref(prog.prog), arr, N.ptr(aggs), 1, s, s, s, s))


def test_join_aggregate_refuses(lib):
    fk = big()
    funcs = np.array([ops.FUNC_COUNT], dtype=np.uint32)
    fargs = (C.c_void_p * 1)(None)
    dk = np.arange(50, dtype=np.uint32)
    q = N.CqlJoinAgg(C.addressof(fk), 1, funcs.ctypes.data, C.addressof(fargs), None, dk.ctypes.data, 50, None, 0, 0, None, 0)
    g, strat = C.c_uint64(), C.c_uint32()
    rows = np.zeros(64, dtype=np.uint64)
    res = np.zeros(64, dtype=np.float64)
    refused(lib, lib.cqlops_join_aggregate(C.byref(q), 64, C.byref(g), N.ptr(rows), N.ptr(res), C.byref(strat)))


def test_sort_and_zone_map_refuse(lib):
    keys = (N.CqlColumn * 1)(big())
    desc = np.zeros(1, dtype=np.uint32)
    out = np.zeros(4, dtype=np.uint32)
    refused(lib, lib.cqlops_sort_rows(keys, 1, N.ptr(desc), None, 0, N.ptr(out), 4))
    zm = np.zeros(4, dtype=np.float64)
    col = big()
    refused(lib, lib.cqlops_zone_map_build(C.byref(col), N.ptr(zm), 2))


def test_rows_at_the_limit_pass_the_guard(lib):
    """4294967294 rows is the largest count taken: the guard lets it through (the call then stops at
    the missing buffer, with a different message)."""
    col = big()
    col.rows = 0xFFFFFFFE
    zm = np.zeros(4, dtype=np.float64)
    assert lib.cqlops_zone_map_build(C.byref(col), N.ptr(zm), 2) == 0
    assert "rows" not in lib.cqlops_last_error().decode() or "at most" not in lib.cqlops_last_error().decode()
