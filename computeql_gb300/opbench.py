"""Per-operator timing: rows/s, GB/s and the kernels behind each operator, on device-resident tables.

    python -m computeql_gb300.opbench [--op NAME ...] [--rows N] [--reps R]

Each operator runs `reps` times after two warm-up calls; the figures are the median wall time of a call
(through the C ABI, inputs resident, results read back) and the CUDA-event time of its kernels. One
JSON line per operator. Inputs are synthetic and seeded (splitmix64 on the device, or numpy), shaped
like the configurations the operators serve:

  sort          ORDER BY one u32 key over `rows` rows
  sort_f64_2    ORDER BY an f64 measure DESC, then a u32 key, over `rows` rows
  sort_subset   ORDER BY an f64 measure over the ~200k rows a filter keeps of a 10M-row table
  fixed         GROUP BY region (50) with SUM/MIN/MAX of a 2-place decimal f64 column
  hash_group    GROUP BY user_id (1M groups) with COUNT and SUM of an f64 measure over 10M rows
  group_small   GROUP BY a key of 5 values with SUM(m0), AVG(m1), MIN(m1), MAX(m1) of two lognormal f64 measures over
                `rows` rows (the one-pass small-key form)
  group_direct  GROUP BY a key of 1M values with COUNT and SUM of a u32 column over `rows` rows (the tables indexed
                by key)
  hll           APPROX_COUNT_DISTINCT(session) over 10M rows (4M distinct)
  hash_join     a 1M-row build side (unique keys) probed by 10M rows, pairs counted
  dense_10k     GROUP BY amount (10k groups) COUNT, SUM(region) over `rows` rows of the seed-0 fact table
  join_small    the join-aggregate probe (join_probe_native) of a 1024-row dim table by `rows` fact rows (random
                keys), COUNT and SUM(amount) per dim row folded into 20 groups: the small build side
  zone_map      the zone map of one u32 column
  batch         512 COUNT+SUM queries over 29 WHERE shapes on a table of 4 u32 + 4 f64 columns, in one shared
                scan (cqlops_batch_filter_aggregate) and, for comparison, one generated kernel per query
"""
from __future__ import annotations

import argparse
import json
import statistics
import time

import numpy as np

from . import build, native, ops, workloads

OPS = ["sort", "sort_f64_2", "sort_subset", "fixed", "hash_group", "group_small", "group_direct", "hll", "hash_join", "join_small",
       "zone_map", "batch", "materialize", "dense_10k"]


def _profile():
    import ctypes as C
    lib = native.load_cuda()
    out = {}
    i = 0
    while True:
        name = C.c_char_p()
        ns = C.c_uint64()
        cnt = C.c_uint64()
        if not lib.cqlcuda_kernel_profile_entry(i, C.byref(name), C.byref(ns), C.byref(cnt)):
            break
        if cnt.value:
            out[name.value.decode()] = (ns.value, cnt.value)
        i += 1
    return out


def _time(fn, reps):
    lib = native.load_cuda()
    fn()
    fn()
    lib.cqlcuda_kernel_profile_reset()
    lib.cqlcuda_kernel_profile_enable(1)
    walls = []
    for _ in range(reps):
        t0 = time.perf_counter()
        fn()
        walls.append((time.perf_counter() - t0) * 1e3)
    lib.cqlcuda_kernel_profile_enable(0)
    prof = _profile()
    kernel_ms = sum(ns for ns, _ in prof.values()) / reps / 1e6
    kernels = {k: {"ms_per_call": ns / reps / 1e6, "launches_per_call": c / reps} for k, (ns, c) in prof.items()}
    return statistics.median(walls), kernel_ms, kernels


def _lognormal_f64(n, seed):
    rng = np.random.default_rng(seed)
    return rng.lognormal(3.0, 1.0, n)


def run(op, rows, reps):
    rng = np.random.default_rng(0)
    if op == "sort":
        key = ops.Column.splitmix(rows, 0, 1, 0, 0)
        perm = np.zeros(rows, dtype=np.uint32)     # the result area kept between calls, as an engine keeps it
        fn = lambda: ops.sort_rows([key], out=perm)
        n, nbytes = rows, rows * 4
    elif op == "sort_f64_2":
        m = ops.Column.from_numpy(_lognormal_f64(rows, 1))
        k = ops.Column.splitmix(rows, 0, 1, 0, 1000)
        perm = np.zeros(rows, dtype=np.uint32)
        fn = lambda: ops.sort_rows([m, k], [1, 0], out=perm)
        n, nbytes = rows, rows * 12
    elif op == "sort_subset":
        total = 10_000_000
        measure = ops.Column.from_numpy(_lognormal_f64(total, 2))
        status = rng.integers(0, 50, total).astype(np.uint32)
        sel_rows = np.nonzero(status == 17)[0].astype(np.uint32)
        sel = ops.DeviceBuffer(sel_rows.nbytes, sel_rows)
        fn = lambda: ops.sort_rows([measure], [0], selection=sel)
        n, nbytes = len(sel_rows), len(sel_rows) * 12
    elif op == "fixed":
        region = ops.Column.splitmix(rows, 0, 3, 0, 50)
        price = ops.Column.from_numpy(rng.integers(0, 10**6, rows) / 100.0)
        fn = lambda: ops.group_dense_fixed(region, [1, 3, 4], [price, price, price])
        n, nbytes = rows, rows * 12
    elif op == "hash_group":
        total = 10_000_000
        user = ops.Column.splitmix(total, 0, 2, 0, 1_000_000)
        measure = ops.Column.from_numpy(_lognormal_f64(total, 3))
        out = ops.HashOutputs(2_000_000, 2)      # the result area kept between calls, as an engine keeps it
        fn = lambda: ops.group_hash([user], [0, 1], [None, measure], group_hint=1_000_000, out=out)
        n, nbytes = total, total * 12
    elif op == "group_small":
        key = ops.Column.splitmix(rows, 7, 1, 0, 5)
        m0 = ops.Column.from_numpy(_lognormal_f64(rows, 4))
        m1 = ops.Column.from_numpy(_lognormal_f64(rows, 5))
        fn = lambda: ops.group_hash([key], [1, 2, 3, 4], [m0, m1, m1, m1], group_hint=5)
        n, nbytes = rows, rows * 20
    elif op == "group_direct":
        key = ops.Column.splitmix(rows, 8, 2, 0, 1_000_000)
        u = ops.Column.splitmix(rows, 8, 2, 1, 1 << 20)
        out = ops.HashOutputs(2_000_000, 2)
        fn = lambda: ops.group_hash([key], [0, 1], [None, u], group_hint=1_000_000, out=out)
        n, nbytes = rows, rows * 8
    elif op == "hll":
        total = 10_000_000
        session = ops.Column.splitmix(total, 0, 2, 1, 4_000_000)
        fn = lambda: ops.group_hash([], [5], [session])
        n, nbytes = total, total * 4
    elif op == "hash_join":
        build_rows, probe_rows = 1_000_000, 10_000_000
        bk = ops.Column.from_numpy(rng.permutation(build_rows).astype(np.uint32))
        pk = ops.Column.splitmix(probe_rows, 0, 1, 0, 1_000_000)
        fn = lambda: ops.hash_join(bk, pk, want_pairs=False)
        n, nbytes = probe_rows, (build_rows + probe_rows) * 4
    elif op == "dense_10k":
        # GROUP BY amount (10k groups) COUNT, SUM(region) over the seed-0 fact table's first `rows` rows
        t = workloads.fact_table(rows)
        fn = lambda: ops.group_dense(t.amount, [ops.FUNC_COUNT, ops.FUNC_SUM], [None, t.region])
        n, nbytes = rows, rows * 8
    elif op == "join_small":
        fk = ops.Column.splitmix(rows, 6, 2, 0, 1024)
        amount = ops.Column.splitmix(rows, 6, 2, 1, 10_000)
        dk = np.arange(1024, dtype=np.uint32)
        seg = (dk % 20).astype(np.float64)
        fn = lambda: ops.join_aggregate(fk, [0, 1], [None, amount], dk, group_values=[seg], strategy=2)
        n, nbytes = rows, rows * 8
    elif op == "materialize":
        # 30 columns of a 10M-row table (20 u32, 10 f64) for the rows of a 1 % filter, read back to the host
        total = 10_000_000
        cols = [ops.Column.splitmix(total, 5, 30, i, 1 << 20) for i in range(20)]
        cols += [ops.Column.from_numpy(rng.random(total)) for _ in range(10)]
        sel_rows = np.sort(rng.choice(total, total // 100, replace=False)).astype(np.uint32)
        fn = lambda: ops.gather_rows(cols, rows=sel_rows)
        n, nbytes = len(sel_rows), len(sel_rows) * (20 * 4 + 10 * 8)
    elif op == "batch":
        return run_batch(rows, reps)
    elif op == "zone_map":
        col = ops.Column.splitmix(rows, 0, 1, 0, 100)
        fn = col.build_zone_map
        n, nbytes = rows, rows * 4
    else:
        raise ValueError(op)
    wall, kernel_ms, kernels = _time(fn, reps)
    return {"op": op, "rows": n, "reps": reps, "wall_ms": wall, "kernel_ms": kernel_ms, "rows_per_s": n / (wall / 1e3),
            "kernel_GBps": nbytes / (kernel_ms / 1e3) / 1e9 if kernel_ms > 0 else None, "bytes": nbytes, "kernels": kernels}


def _batch_queries(count, shape_count, seed):
    """WHERE shapes drawn like the reference's per-query kernel benchmark (pc_random_shape,
    src/tests/bench_perquery_compile.c:238-258): 1-8 range comparisons over the 8 columns, one in four
    joined by OR, one parenthesised pair when there are 4 or more; each query a shape with new literals."""
    u32, f64 = ["u0", "u1", "u2", "u3"], ["d0", "d1", "d2", "d3"]
    cols = u32 + f64
    srng = np.random.default_rng(seed)
    states = [int(srng.integers(0, 2**63)) for _ in range(shape_count)]
    qrng = np.random.default_rng(seed + 1)

    def lit(c):
        return int(qrng.integers(0, 1 << 16)) if c[0] == "u" else round(float(qrng.random()), 6)

    def shape(state):
        r = np.random.default_rng(state)
        n = 1 + int(r.integers(0, 8))
        leaves, join = [], []
        for _ in range(n):
            c = cols[int(r.integers(0, len(cols)))]
            upper, inclusive = bool(r.integers(0, 2)), bool(r.integers(0, 2))
            op = ("<=" if inclusive else "<") if upper else (">=" if inclusive else ">")
            leaves.append(f"({op} {c} {lit(c)!r})")
            join.append(int(r.integers(0, 4)) == 0)
        items, i = [], 0
        group = int(r.integers(0, n - 2)) if n >= 4 else None
        if group is not None:
            join[group] = not join[group + 1]
        while i < n:
            if i == group:
                items += [f"({'or' if join[i] else 'and'} {leaves[i]} {leaves[i + 1]})", "or" if join[i + 1] else "and"]
                i += 2
            else:
                items += [leaves[i], "or" if join[i] else "and"]
                i += 1
        items = items[:-1]
        terms, cur = [], [items[0]]
        for k in range(1, len(items), 2):
            if items[k] == "and":
                cur.append(items[k + 1])
            else:
                terms.append(cur)
                cur = [items[k + 1]]
        terms.append(cur)

        def chain(o, xs):
            out = xs[0]
            for x in xs[1:]:
                out = f"({o} {out} {x})"
            return out
        return chain("or", [chain("and", t) for t in terms])

    return [(shape(states[q % shape_count]), f64[q % 4]) for q in range(count)]


def run_batch(rows, reps):
    rng = np.random.default_rng(4)
    cols = {f"u{i}": ops.Column.splitmix(rows, 4, 8, i, 1 << 16) for i in range(4)}
    cols.update({f"d{i}": ops.Column.from_numpy(rng.random(rows)) for i in range(4)})
    qs = _batch_queries(512, 29, 9)
    progs = [ops.Program(w, cols) for w, _ in qs]
    sums = [s for _, s in qs]
    best = None
    tuning = {}
    for rpt in (0, 4, 8, 16):
        # the tuning knob: the shared-memory tile form (0) or the register form with 4, 8 or 16 rows per
        # thread; the fastest kept
        wall, kernel_ms, kernels = _time(lambda: ops.batch_aggregate(progs, sums, rpt), reps)
        tuning["tile" if rpt == 0 else f"rows_per_thread_{rpt}"] = round(wall, 3)
        if best is None or wall < best[1]:
            best = (rpt, wall, kernel_ms, kernels)
    # one generated kernel per (shape, summed column), 116 here: past the default cap of 64 they would be evicted
    # and compiled again in turn, so the cap is raised for this path
    lib = native.load_cuda()
    lib.cqlcuda_set_generated_kernel_cap(256)
    one_wall, one_kernel, _ = _time(lambda: [ops.fused_aggregate(p, [s]) for p, s in zip(progs, sums)], max(1, reps // 2))
    lib.cqlcuda_set_generated_kernel_cap(64)
    # the autotuner: its trial runs (one per candidate form) first, then its pick
    auto = ops.CQLOPS_BATCH_AUTOTUNE
    for _ in range(8):
        ops.batch_aggregate(progs, sums, auto)
    auto_wall, auto_kernel, _ = _time(lambda: ops.batch_aggregate(progs, sums, auto), reps)
    auto_form = native.load_ops().cqlops_batch_last_form()
    persistent = _persistent_ab(progs, sums, best[0] if best[0] else 8, reps)
    graphs = _graph_ab(reps)
    nbytes = rows * (4 * 4 + 4 * 8)
    return {"op": "batch", "rows": rows, "queries": len(qs), "shapes": 29, "reps": reps, "rows_per_thread": best[0], "tuning_wall_ms": tuning,
            "wall_ms": best[1], "kernel_ms": best[2], "rows_per_s": len(qs) * rows / (best[1] / 1e3),
            "kernel_GBps": nbytes / (best[2] / 1e3) / 1e9, "bytes": nbytes, "kernels": best[3],
            "one_at_a_time_wall_ms": one_wall, "one_at_a_time_kernel_ms": one_kernel, "speedup_wall": one_wall / best[1],
            "autotuned_wall_ms": auto_wall, "autotuned_kernel_ms": auto_kernel,
            "autotuned_form": {"rows_per_thread": auto_form & 0xff, "block": 256 * max(1, (auto_form >> 8) & 0xff)} if auto_form & 0xff
            else {"form": "tile"}, "persistent": persistent, "plan_graphs": graphs}


def _persistent_ab(progs, sums, rows_per_thread, reps):
    """The 512 queries as a catalog batch launched (two launches: 384 + 128 queries) and through the persistent
    scan (two runs), wall time; the launched ones first - an allocation elsewhere waits for a running
    persistent kernel."""
    cat = ops.BatchCatalog()
    halves = [(progs[:384], sums[:384]), (progs[384:], sums[384:])]
    for p, s in halves:
        cat.aggregate(p, s, rows_per_thread)
    walls = []
    want = None
    for _ in range(reps):
        t0 = time.perf_counter()
        want = [cat.aggregate(p, s, rows_per_thread)[:2] for p, s in halves]
        walls.append((time.perf_counter() - t0) * 1e3)
    with ops.PersistentScan(cat, progs, rows_per_thread=rows_per_thread, idle_us=500_000) as ps:
        for p, s in halves:
            ps.run(p, s)
        pwalls = []
        same = True
        for _ in range(reps):
            t0 = time.perf_counter()
            got = [ps.run(p, s) for p, s in halves]
            pwalls.append((time.perf_counter() - t0) * 1e3)
            same = same and all(np.array_equal(g[0], w[0]) and np.array_equal(g[1].view(np.uint64), w[1].view(np.uint64))
                                for g, w in zip(got, want))
        st = ps.stats()
    return {"rows_per_thread": rows_per_thread, "launched_wall_ms": statistics.median(walls), "persistent_wall_ms": statistics.median(pwalls),
            "identical": bool(same), **st}


def _graph_ab(reps):
    """Plan graphs on and off: batches of 8 queries of the batched workload's shapes over a 1M-row table
    (where the launches, not the scan, are most of a batch), wall time without profiling."""
    lib = native.load_cuda()
    rng = np.random.default_rng(5)
    n = 1_000_000
    cols = {f"u{i}": ops.Column.splitmix(n, 5, 8, i, 1 << 16) for i in range(4)}
    cols.update({f"d{i}": ops.Column.from_numpy(rng.random(n)) for i in range(4)})
    qs = _batch_queries(8, 4, 13)
    progs = [ops.Program(w, cols) for w, _ in qs]
    sums = [s for _, s in qs]

    def wall(count):
        fn = lambda: ops.batch_aggregate(progs, sums, 8)
        fn()
        fn()
        walls = []
        for _ in range(count):
            t0 = time.perf_counter()
            fn()
            walls.append((time.perf_counter() - t0) * 1e3)
        return statistics.median(walls)

    count = max(20, reps * 10)
    on = wall(count)
    lib.cqlcuda_graph_enable(0)
    off = wall(count)
    lib.cqlcuda_graph_enable(1)
    return {"rows": n, "queries": len(qs), "graph_wall_ms": round(on, 4), "eager_wall_ms": round(off, 4)}


def main(argv=None):
    ap = argparse.ArgumentParser()
    ap.add_argument("--op", action="append", choices=OPS)
    ap.add_argument("--rows", type=int, default=100_000_000)
    ap.add_argument("--reps", type=int, default=5)
    args = ap.parse_args(argv)
    build.build()
    native.init()
    for op in args.op or OPS:
        print(json.dumps(run(op, args.rows, args.reps)), flush=True)


if __name__ == "__main__":
    main()
