"""The batched scan's generated kernel (cqlops_batch_source), built and NVRTC-compiled without a GPU."""
import numpy as np
import pytest

from tests.batch_workload import F64, U32, queries


@pytest.fixture(scope="module")
def ops():
    from computeql_gb300 import build, ops as o
    build.build()
    return o


def columns(ops, rows=1000):
    cols = {n: ops.Column(ops.TYPE_U32, rows, zone=(0.0, 65535.0)) for n in U32}
    cols.update({n: ops.Column(ops.TYPE_F64, rows, zone=(0.0, 1.0)) for n in F64})
    return cols


@pytest.mark.parametrize("rows_per_thread", [0, 4, 8, 16])
def test_source_compiles(ops, rows_per_thread):
    cols = columns(ops)
    qs = queries(120, 29, 3)
    progs = [ops.Program(w, cols) for w, _ in qs]
    src, shapes = ops.batch_source(progs, [s for _, s in qs], rows_per_thread)
    assert shapes == 29
    assert src.count("#define CQL_SHAPE_") == 29
    ok, log = ops.compile_check(src)
    assert ok, log


def test_queries_of_one_shape_share_its_predicate(ops):
    cols = columns(ops)
    qs = [(f"(and (< u0 {k}) (>= d1 0.{k}))", "d0") for k in range(1, 50)]
    progs = [ops.Program(w, cols) for w, _ in qs]
    src, shapes = ops.batch_source(progs, [s for _, s in qs])
    assert shapes == 1
    # the literals are per-query thresholds, not in the source
    assert "#define CQL_SHAPE_0(k) ((cql_bi(&T0, r0[k]) & cql_bk(&T1, kd5[k])))" in src


def test_strings_are_refused(ops):
    cols = columns(ops)
    cols["s"] = ops.Column(ops.TYPE_STRING8, 1000)
    progs = [ops.Program("(= s 'x')", cols)]
    with pytest.raises(ops.OpError):
        ops.batch_source(progs, [None])


def test_tile_form_sizes_its_shared_memory(ops):
    """The tile form stages 1024 rows when they fit in 72 KB with the accumulators, else 512, and asks for
    as many CTAs per SM as 227 KB holds (at most 8)."""
    cols = columns(ops)
    qs = queries(64, 8, 5)
    progs = [ops.Program(w, cols) for w, _ in qs]
    src, _ = ops.batch_source(progs, [s for _, s in qs], 0)
    head = src.splitlines()[0]
    assert head.startswith("// cql: block=256 smem=")
    smem = int(head.split("smem=")[1].split()[0])
    per_sm = int(head.split("per_sm=")[1].split()[0])
    assert "const u32 TILE = 512u" in src or "const u32 TILE = 1024u" in src
    assert smem <= 227 * 1024 and 1 <= per_sm <= 8 and per_sm * (smem + 1024) <= 227 * 1024


def cube_columns(ops, rows=1000):
    return {"region": ops.Column(ops.TYPE_U32, rows, zone=(0.0, 49.0)), "flag": ops.Column(ops.TYPE_U32, rows, zone=(0.0, 99.0)),
            "status": ops.Column(ops.TYPE_I32, rows, zone=(-3.0, 5.0)), "amount": ops.Column(ops.TYPE_U32, rows, zone=(0.0, 9999.0)),
            "v": ops.Column(ops.TYPE_F64, rows, zone=(0.0, 1e6))}


def test_cube_sources_compile(ops):
    """The cube kernels of a mixed batch NVRTC-compile for sm_103a: the answers and every table pass (the
    {flag, region} table with two sums fills a pass of its own). Only the small-range integer shapes go to
    the cube (the f64 comparison stays on the scan)."""
    cols = cube_columns(ops)
    qs = [("(< flag 7)", None), ("(= region 3)", "amount"), ("(and (< flag 9) (and (>= region 4) (< region 9)))", "v"),
          ("(and (>= amount 100) (< amount 900))", None), ("(and (or (= region 1) (= region 2)) (>= flag 50))", "amount"),
          ("(and (<= status 2) (> flag 10))", "status"), ("(> v 3.5)", "amount")]
    progs = [ops.Program(w, cols) for w, _ in qs]
    sums = [s for _, s in qs]
    src, n = ops.batch_cube_source(progs, sums, 0)
    assert n == 6
    ok, log = ops.compile_check(src)
    assert ok, log
    passes = 0
    while True:
        try:
            src, _ = ops.batch_cube_source(progs, sums, 1 + passes)
        except ops.OpError:
            break
        ok, log = ops.compile_check(src)
        assert ok, log
        passes += 1
    assert passes == 2


def test_no_cube_for_wide_or_float_columns(ops):
    cols = cube_columns(ops)
    progs = [ops.Program(w, cols) for w in ("(> v 3.5)", "(< v 1.0)")]
    with pytest.raises(ops.OpError):
        ops.batch_cube_source(progs, [None, None], 0)


@pytest.mark.parametrize("rows_per_thread", [4, 8, 16])
def test_persistent_source_compiles(ops, rows_per_thread):
    """The persistent form: the scan as a device function adding into accumulators, its one-pass entry and
    the queue loop, every wait bounded by the idle limit (a time read from the global timer)."""
    cols = columns(ops)
    qs = queries(120, 29, 3)
    progs = [ops.Program(w, cols) for w, _ in qs]
    src, shapes = ops.batch_source(progs, [s for _, s in qs], rows_per_thread | 0x10000)
    assert shapes == 29
    assert "cql_persist(CqlLaunch p)" in src and "cql_main(CqlLaunch a)" in src
    assert "cql_now() - t0 > idle_ns" in src and "fence.acq_rel.gpu" in src
    ok, log = ops.compile_check(src)
    assert ok, log
