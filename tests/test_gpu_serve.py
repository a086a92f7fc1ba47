"""The served form on the GPU: the shape catalog, concurrent lanes and the server (include/cqlserve.h).

A served result must equal the same query run alone:
  - counts bit for bit against the oracle's restatement of the bytecode interpreter;
  - a shared scan's SUM bit for bit against the same query in a shared scan of its own (the sums are
    exact sums of scaled integers, independent of the other queries) and within 1e-12 of math.fsum;
  - whole-column aggregates and dense GROUP BY bit for bit against the operator called directly.
Admission is checked with requests that hold no device memory but declare a footprint.
"""
import math
import threading
import time

import numpy as np
import pytest

from tests.batch_workload import F64, U32, shapes, table
from tests.where_shapes import oracle_mask

pytestmark = pytest.mark.gpu

ROWS = 1_000_003


@pytest.fixture(scope="module")
def env(gpu):
    from computeql_gb300 import ops
    arrays = table(ROWS, 21)
    arrays["k"] = np.random.default_rng(22).integers(0, 50, ROWS).astype(np.uint32)
    cols = {n: ops.Column.from_numpy(a) for n, a in arrays.items()}
    return ops, arrays, cols


def _queries(count, shape_count, seed):
    makers = shapes(shape_count, seed)
    rng = np.random.default_rng(seed + 100)
    out = []
    for q in range(count):
        where = makers[q % shape_count](rng)
        out.append((where, F64[q % 4] if q % 3 else None))
    return out


def _exact_sum(arrays, prog, scol):
    m = oracle_mask(prog, arrays).astype(bool)
    return int(m.sum()), (math.fsum(arrays[scol][m]) if scol else 0.0)


def test_catalog_matches_the_plain_batch_and_reuses_its_kernel(env):
    ops, arrays, cols = env
    from computeql_gb300 import native
    lib = native.load_cuda()
    cat = ops.BatchCatalog()
    first = _queries(48, 6, 3)
    progs = [ops.Program(w, cols) for w, _ in first]
    sums = [s for _, s in first]
    c1, s1, _ = cat.aggregate(progs, sums)
    c0, s0, _ = ops.batch_aggregate(progs, sums)
    assert np.array_equal(c1, c0)
    assert np.array_equal(s1, s0)
    assert cat.shapes == 6
    # a later batch of two of the known shapes with new literals: no new kernel
    compiles = native.C.c_uint64()
    lib.cqlcuda_generated_kernel_stats(native.C.byref(compiles), None)
    before = compiles.value
    second = [q for i, q in enumerate(_queries(60, 6, 3)) if i % 6 in (1, 4)][:10]
    progs2 = [ops.Program(w, cols) for w, _ in second]
    c2, s2, _ = cat.aggregate(progs2, [s for _, s in second])
    lib.cqlcuda_generated_kernel_stats(native.C.byref(compiles), None)
    assert compiles.value == before
    assert cat.shapes == 6
    for i, (w, scol) in enumerate(second):
        cnt, exact = _exact_sum(arrays, progs2[i], scol)
        assert c2[i] == cnt, w
        if scol:
            assert abs(s2[i] - exact) <= 1e-12 * max(abs(exact), 1e-300), w
    cat.close()


def test_lanes_run_operators_concurrently(env):
    ops, arrays, cols = env
    from computeql_gb300 import native
    lib = native.load_cuda()
    qs = _queries(12, 4, 5)
    progs = [ops.Program(w, cols) for w, _ in qs]
    serial = [ops.fused_aggregate(p, [s] if s else []) for p, (_, s) in zip(progs, qs)]
    serial_g = ops.aggregate_global([cols["u0"], cols["d1"]])
    serial_d = ops.group_dense(cols["k"], [ops.FUNC_COUNT, ops.FUNC_SUM, ops.FUNC_MAX], [None, cols["u1"], cols["u2"]])
    results = {}
    errors = []

    def worker(t):
        try:
            assert lib.cqlcuda_thread_lane_begin(f"t{t}".encode())
            out = []
            for _ in range(3):
                out.append([ops.fused_aggregate(p, [s] if s else []) for p, (_, s) in zip(progs, qs)])
                out.append(ops.aggregate_global([cols["u0"], cols["d1"]]))
                out.append(ops.group_dense(cols["k"], [ops.FUNC_COUNT, ops.FUNC_SUM, ops.FUNC_MAX], [None, cols["u1"], cols["u2"]]))
            results[t] = out
        except Exception as e:   # reported on the main thread
            errors.append(e)
        finally:
            lib.cqlcuda_thread_lane_end()

    threads = [threading.Thread(target=worker, args=(t,)) for t in range(4)]
    for th in threads:
        th.start()
    for th in threads:
        th.join()
    assert not errors, errors
    for t in range(4):
        for r in range(3):
            assert results[t][3 * r] == serial
            assert results[t][3 * r + 1] == serial_g
            d = results[t][3 * r + 2]
            assert d[0] == serial_d[0]
            for a, b in zip(d[1:], serial_d[1:]):
                assert np.array_equal(a, b)


@pytest.mark.parametrize("workers,fuse", [(3, True), (1, False), (4, False)])
def test_served_results_equal_each_query_alone(env, workers, fuse):
    ops, arrays, cols = env
    qs = _queries(120, 8, 9)
    with ops.Server(workers=workers, fuse=fuse) as sv:
        t = sv.add_table(cols)
        progs = [t.program(w) for w, _ in qs]
        sv.prepare(t, progs[:8], [s for _, s in qs[:8]])
        reqs = [None] * len(qs)
        extra = []

        def submitter(part):
            for i in range(part, len(qs), 4):
                reqs[i] = sv.filter_agg(t, progs[i], qs[i][1])
                if i % 20 == 0:
                    extra.append(("g", sv.agg_global(t, ["u0", "d1", "k"])))
                    extra.append(("d", sv.group_dense(t, "k", [ops.FUNC_COUNT, ops.FUNC_SUM, ops.FUNC_MIN], [None, "u1", "u2"])))

        threads = [threading.Thread(target=submitter, args=(p,)) for p in range(4)]
        for th in threads:
            th.start()
        for th in threads:
            th.join()
        for r in reqs:
            assert r.wait(60000)
        for _, r in extra:
            assert r.wait(60000)
        stats = sv.stats()
        fused = [r.fused for r in reqs]
    assert all(r.ok for r in reqs), [r.error for r in reqs if not r.ok][:3]
    alone_c, alone_s, _ = ops.batch_aggregate(progs, [s for _, s in qs]) if fuse else (None, None, None)
    for i, (w, scol) in enumerate(qs):
        cnt, exact = _exact_sum(arrays, progs[i], scol)
        assert reqs[i].count == cnt, w
        if scol:
            assert abs(reqs[i].sum - exact) <= 1e-12 * max(abs(exact), 1e-300), w
            if fuse:
                assert reqs[i].sum == alone_s[i], w     # the shared scan's sum does not depend on its company
    g_ref = ops.aggregate_global([cols["u0"], cols["d1"], cols["k"]])
    d_ref = ops.group_dense(cols["k"], [ops.FUNC_COUNT, ops.FUNC_SUM, ops.FUNC_MIN], [None, cols["u1"], cols["u2"]])
    for kind, r in extra:
        assert r.ok, r.error
        if kind == "g":
            assert (list(r.req.sum[:3]), list(r.req.min[:3]), list(r.req.max[:3])) == g_ref
        else:
            got = r.group_result()
            assert got[0] == d_ref[0]
            for a, b in zip(got[1:], d_ref[1:]):
                assert np.array_equal(a, b)
    assert stats["completed"] == len(qs) + len(extra)
    assert stats["failed"] == 0
    assert stats["in_flight_bytes"] == 0
    if fuse:
        assert stats["scans"] <= len(qs)
        assert stats["fused_requests"] == len(qs)
    else:
        assert max(fused) == 1 and stats["scans"] == 0


def test_fused_requests_share_a_scan_when_they_queue(env):
    ops, arrays, cols = env
    qs = _queries(64, 4, 13)
    with ops.Server(workers=1, fuse=True) as sv:
        t = sv.add_table(cols)
        progs = [t.program(w) for w, _ in qs]
        sv.prepare(t, progs[:4], [s for _, s in qs[:4]])
        # hold the only worker so that the queries queue behind it
        gate = threading.Event()
        hold = sv.call(lambda: gate.wait(30) or True)
        reqs = [sv.filter_agg(t, p, s) for p, (_, s) in zip(progs, qs)]
        gate.set()
        assert hold.wait(60000) and hold.ok
        for r in reqs:
            assert r.wait(60000)
        stats = sv.stats()
    assert all(r.fused == len(qs) for r in reqs), [r.fused for r in reqs]
    assert stats["scans"] == 1 and stats["max_fused"] == len(qs)
    for i, (w, scol) in enumerate(qs):
        cnt, _ = _exact_sum(arrays, progs[i], scol)
        assert reqs[i].count == cnt, w


def test_admission_keeps_planned_memory_within_budget(gpu):
    from computeql_gb300 import ops
    mb = 1 << 20
    running = [0]
    peak = [0]
    lock = threading.Lock()

    def job():
        with lock:
            running[0] += 1
            peak[0] = max(peak[0], running[0])
        time.sleep(0.02)
        with lock:
            running[0] -= 1
        return True

    with ops.Server(workers=4, fuse=True, memory_budget=100 * mb) as sv:
        big = [sv.call(job, footprint=60 * mb) for _ in range(6)]
        for r in big:
            assert r.wait(60000) and r.ok
        assert peak[0] == 1                    # two 60 MB requests never run together under 100 MB
        peak[0] = 0
        small = [sv.call(job, footprint=30 * mb) for _ in range(12)]
        for r in small:
            assert r.wait(60000) and r.ok
        assert 2 <= peak[0] <= 3               # three fit, a fourth does not
        too_big = sv.call(job, footprint=101 * mb)
        assert too_big.wait(60000)
        assert too_big.status == -1 and "budget" in too_big.error
        stats = sv.stats()
    assert stats["peak_in_flight_bytes"] <= 100 * mb
    assert stats["admission_waits"] > 0
    assert stats["failed"] == 1


def test_bad_requests_fail_at_submit(env):
    ops, arrays, cols = env
    from computeql_gb300 import native
    with ops.Server(workers=1) as sv:
        t = sv.add_table(cols)
        req = native.CqlServeRequest()
        req.kind = 99
        req.table = t.index
        r = ops.ServeRequest(sv, req, ())
        assert native.load_ops().cqlserve_submit(sv.h, native.C.byref(req)) == 0
        assert r.status == -1 and "unknown" in r.error
        req2 = native.CqlServeRequest()
        req2.kind = ops.SERVE_AGG_GLOBAL
        req2.table = 7
        req2.column_count = 1
        assert native.load_ops().cqlserve_submit(sv.h, native.C.byref(req2)) == 0
        assert b"no such table" in req2.error


def test_identical_requests_share_one_run(env):
    ops, arrays, cols = env
    with ops.Server(workers=1, fuse=True) as sv:
        t = sv.add_table(cols)
        gate = threading.Event()
        hold = sv.call(lambda: gate.wait(30) or True)
        groups = [sv.group_dense(t, "k", [ops.FUNC_COUNT, ops.FUNC_SUM, ops.FUNC_MAX], [None, "u1", "u2"]) for _ in range(5)]
        globs = [sv.agg_global(t, ["u0", "d1"]) for _ in range(3)]
        other = sv.agg_global(t, ["u3"])
        gate.set()
        for r in [hold] + groups + globs + [other]:
            assert r.wait(60000) and r.ok, r.error
        stats = sv.stats()
    d_ref = ops.group_dense(cols["k"], [ops.FUNC_COUNT, ops.FUNC_SUM, ops.FUNC_MAX], [None, cols["u1"], cols["u2"]])
    for r in groups:
        got = r.group_result()
        assert got[0] == d_ref[0] and r.fused == 5
        for a, b in zip(got[1:], d_ref[1:]):
            assert np.array_equal(a, b)
    g_ref = ops.aggregate_global([cols["u0"], cols["d1"]])
    for r in globs:
        assert (list(r.req.sum[:2]), list(r.req.min[:2]), list(r.req.max[:2])) == g_ref and r.fused == 3
    assert other.fused == 1 and other.req.sum[0] == ops.aggregate_global([cols["u3"]])[0][0]
    assert stats["merged_requests"] == 4 + 2


def test_join_and_sort_requests_equal_their_operators(gpu):
    """The served mix's join and ORDER BY templates run as native call requests on the workers' lanes; in a
    mix with filter/aggregate and group-by requests each answers what its operator answers alone."""
    from computeql_gb300 import ops, workloads
    import numpy as np
    n = 2_000_003
    f = workloads.fact_table(n, seed=5)
    cols = {"region": f.region, "amount": f.amount, "flag": f.flag}
    d50, d1m = workloads.dim_tables()
    seg = d1m["seg"].astype(np.float64)
    kept = np.nonzero(d50["name_id"] == 4)[0]
    want_j50 = ops.join_aggregate(f.region, [ops.FUNC_COUNT, ops.FUNC_SUM], [None, f.amount], d50["k"], dim_rows=kept)
    want_j1m = ops.join_aggregate(f.amount, [ops.FUNC_SUM, ops.FUNC_COUNT], [f.amount, None], d1m["k"], group_values=[seg])
    cnt, sel = ops.scan_simple([f.flag], [(0, ops.CMP_EQ, 7)], want_rows=True)
    sel_buf = ops.DeviceBuffer(len(sel) * 4, sel)
    want_sort = ops.sort_rows([f.amount], [1], selection=sel_buf, count=len(sel))[:100]
    with ops.Server(workers=3, fuse=True) as sv:
        table = sv.add_table(cols)
        reqs = []
        for i in range(6):
            reqs.append(("j50", sv.join(f.region, [ops.FUNC_COUNT, ops.FUNC_SUM], [None, f.amount], d50["k"], dim_rows=kept,
                                        dim_key_col=d50["k_col"])))
            reqs.append(("j1m", sv.join(f.amount, [ops.FUNC_SUM, ops.FUNC_COUNT], [f.amount, None], d1m["k"], group_values=[seg],
                                        dim_key_col=d1m["k_col"], dim_group_col=d1m["seg_col"])))
            reqs.append(("sort", sv.sort([f.flag, f.amount], [(0, ops.CMP_EQ, 7)], 1, True, 100, n // 50)))
            reqs.append(("filter", sv.filter_agg(table, table.program(f"(< flag {10 + i})"), "amount")))
            reqs.append(("group", sv.group_dense(table, "region", [ops.FUNC_COUNT], [None])))
        for kind, r in reqs:
            assert r.wait(60_000) and r.ok, (kind, r.error)
            if kind in ("j50", "j1m"):
                ctx = r._keep["ctx"]
                want = want_j50 if kind == "j50" else want_j1m
                g = ctx.groups
                assert g == want["groups"]
                assert np.array_equal(r._keep["rows"][:g], want["dim_row"])
                assert np.array_equal(r._keep["res"][: g * 2].reshape(g, 2), want["results"])
            elif kind == "sort":
                assert r._keep["ctx"].count == cnt
                assert np.array_equal(r._keep["out"], want_sort)
