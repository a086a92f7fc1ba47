"""Benchmark: warm rows/s and % of HBM peak per query on the 1B-row table (one GB300).

A step runs the query suite of the 1B-row configuration once over a warm, device-resident table:
  q1 SELECT SUM(amount), MIN(amount), MAX(amount)                  aggregate_global_native
  q2 SELECT COUNT(*) WHERE flag < 2                                scan_simple (count only)
  q3 SELECT region, SUM(amount), COUNT(*) GROUP BY region         aggregate_dense_native, 50 groups
  q4 SELECT amount, COUNT(*), SUM(region) GROUP BY amount         aggregate_dense_native, 10k groups
  q5 SELECT id, ... WHERE id = k (a random k)                      scan_simple on the id sequence
  q6 SELECT COUNT(*), SUM(amount) FROM fact JOIN dim50 ON region = dim50.k WHERE dim50.name_id = 3
                                                                    join_probe_native (dense core)
  q7 SELECT seg, SUM(amount), COUNT(*) FROM fact JOIN dim1M ON amount % 1000000 = dim1M.k GROUP BY seg
                                                                    join_probe_native (dense core)
value = (queries x rows) / suite time, on the device (CUDA events around the step, inputs larger
than L2). `e2e` runs the same suite through the C ABI from pinned HOST buffers: every step uploads the
columns the queries read and reads the results back. `roofline` is the dominant kernel's algorithmic
bytes per launch over its CUDA-event duration. `cpu_baseline` times the oracle's CPU restatement of
the reference's operators on a bounded sample with all host cores.

--impl reference times that CPU restatement alone (the reference's own CPU operator path does not
build on Linux: it is a Win32-only unity build).
"""
from __future__ import annotations

import argparse
import json
import os
import statistics
import subprocess
import sys
import tempfile
import time

ROOT = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, ROOT)

METRIC = "warm rows/s and % HBM peak per query at 1B rows"
UNIT = "rows/s"
PEAKS_FILE = os.path.join(ROOT, "MEASURED_PEAKS.json")
FALLBACK_HBM_GBS = 6800.0
CPU_SAMPLE_ROWS = 100_000_000
N_QUERIES = 7


def hbm_peak():
    try:
        with open(PEAKS_FILE) as f:
            return float(json.load(f)["hbm_gbs"]), "measured"
    except Exception:
        return FALLBACK_HBM_GBS, "fallback"


class Clocks:
    """nvidia-smi sampling during the timed region."""

    def __init__(self):
        self.proc = None
        self.path = None

    def start(self):
        try:
            fd, self.path = tempfile.mkstemp(suffix=".csv")
            os.close(fd)
            q = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,clocks_event_reasons.hw_slowdown,"
                 "clocks_event_reasons.hw_thermal_slowdown,clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")
            self.proc = subprocess.Popen(["nvidia-smi", f"--query-gpu={q}", "--format=csv,noheader,nounits", "-lms", "100"],
                                         stdout=open(self.path, "w"), stderr=subprocess.DEVNULL)
            time.sleep(0.3)
        except Exception:
            self.proc = None

    def stop(self, device_index=0):
        if not self.proc:
            return None
        self.proc.terminate()
        try:
            self.proc.wait(timeout=5)
        except Exception:
            self.proc.kill()
        sm, mx, reasons = [], None, set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        with open(self.path) as f:
            for line in f:
                p = [x.strip() for x in line.split(",")]
                if len(p) < 9 or p[0] != str(device_index):
                    continue
                try:
                    sm.append(float(p[1]))
                    mx = float(p[2])
                except ValueError:
                    continue
                for name, v in zip(names, p[5:9]):
                    if v.lower() == "active":
                        reasons.add(name)
        os.unlink(self.path)
        if not sm:
            return None
        return {"sm_mhz": statistics.median(sm), "sm_max_mhz": mx, "reasons": sorted(reasons), "samples": len(sm)}


def make_queries(ops, t, rng_key, dims):
    """The suite as (name, algorithmic bytes, callable)."""
    import numpy as np
    n = t.rows
    k = int(rng_key)
    d50, d1m = dims
    seg_values = d1m["seg"].astype(np.float64)

    def q1():
        return ops.aggregate_global([t.amount])

    def q2():
        return ops.scan_simple([t.flag], [(0, ops.CMP_LT, 2)])

    def q3():
        return ops.group_dense(t.region, [ops.FUNC_SUM, ops.FUNC_COUNT], [t.amount, None])

    def q4():
        return ops.group_dense(t.amount, [ops.FUNC_COUNT, ops.FUNC_SUM], [None, t.region])

    def q5():
        return ops.scan_simple([t.id], [(0, ops.CMP_EQ, k)], want_rows=True, max_rows=16)

    # the dimension tables are resident on the device too: the joins' dim-row passes run there
    def q6():
        kept = np.nonzero(d50["name_id"] == 3)[0]          # the dimension filter (50 rows)
        return ops.join_aggregate(t.region, [ops.FUNC_COUNT, ops.FUNC_SUM], [None, t.amount], d50["k"], dim_rows=kept,
                                  dim_key_col=d50.get("k_col"))

    def q7():
        # amount < 10000, so amount % 1000000 is amount itself
        return ops.join_aggregate(t.amount, [ops.FUNC_SUM, ops.FUNC_COUNT], [t.amount, None], d1m["k"],
                                  group_values=[seg_values], dim_key_col=d1m.get("k_col"), dim_group_col=d1m.get("seg_col"))

    # algorithmic bytes: the distinct stored columns a query reads x rows x 4 B. The id lookup reads
    # none: id is a sequence (never stored) and its zone map keeps one 8192-row chunk, latency-bound.
    return [("sum_min_max_amount", 4 * n, q1), ("count_flag_lt_2", 4 * n, q2), ("group_by_region", 8 * n, q3),
            ("group_by_amount_10k", 8 * n, q4), ("point_lookup_id", 0, q5), ("join_dim50_filtered", 8 * n, q6),
            ("join_dim1m_group_by_seg", 4 * n, q7)]


def parity_checks(ops, t, queries, dims, key):
    """The suite's answers, checked once outside the timed region; returns (status, checks run).

    1. Seed-0 table: every query's result against another kernel path over the same columns - the
       dense group-bys' totals against the global aggregate, the filter count against a dense
       GROUP BY flag, the dim50 join against GROUP BY region's groups of the kept regions, the dim1M
       join grouped by seg against GROUP BY amount folded through dim1M's seg, and the point lookup's
       row against its key.
    2. The reference's closed-form scale table at the same size (src/tests/scale/bench_select_scale.c:
       38-56, filled on the device) against the reference's own known answers (:97-167, cases
       :1085-1170): SUM/MIN/MAX, the 0.1 % and 2 % filters, the id lookup, GROUP BY region, GROUP BY
       amount, the filtered join to its 50-row table and the join to its 10k-row table grouped by
       category.
    """
    import numpy as np
    from tests import closed_form as cf
    n = t.rows
    d50, d1m = dims
    got = {name: q() for name, _, q in queries}
    checks = []

    def check(name, ok):
        checks.append(name)
        if not ok:
            raise AssertionError(name)

    try:
        s, mn, mx = got["sum_min_max_amount"]
        mk3, c3, s3, _, _ = got["group_by_region"]
        check("group_by_region counts total rows", int(c3.sum()) == n)
        check("group_by_region sums total SUM(amount)", float(s3[:, 0].sum()) == s[0])
        mk4, c4, s4, _, _ = got["group_by_amount_10k"]
        rs, _, _ = ops.aggregate_global([t.region])
        check("group_by_amount counts total rows", int(c4.sum()) == n)
        check("group_by_amount sums total SUM(region)", float(s4[:, 1].sum()) == rs[0])
        present = np.nonzero(c4)[0]
        check("MIN/MAX(amount) are the extreme amount groups", (mn[0], mx[0]) == (float(mk4 + present[0]), float(mk4 + present[-1])))
        check("amount groups are their values x counts", float((c4.astype(np.float64) * (mk4 + np.arange(len(c4)))).sum()) == s[0])
        mkf, cf_, _, _, _ = ops.group_dense(t.flag, [ops.FUNC_COUNT], [None])
        check("count flag < 2 equals GROUP BY flag's groups 0 and 1", got["count_flag_lt_2"][0] == int(cf_[: 2 - int(mkf)].sum()))
        cnt, rows = got["point_lookup_id"]
        check("point lookup finds its one row", cnt == 1 and list(rows) == [key])
        kept = np.nonzero(d50["name_id"] == 3)[0]
        r6 = got["join_dim50_filtered"]["results"]
        check("dim50 join equals GROUP BY region over the kept regions",
              (r6[0, 0], r6[0, 1]) == (float(c3[kept - mk3].sum()), float(s3[kept - mk3, 0].sum())))
        r7 = got["join_dim1m_group_by_seg"]
        amounts = mk4 + np.arange(len(c4))
        seg_of = d1m["seg"][amounts % 1_000_000]
        for g in range(r7["groups"]):
            seg = d1m["seg"][int(r7["dim_row"][g])]
            sel = seg_of == seg
            want = (float((c4[sel].astype(np.float64) * amounts[sel]).sum()), float(c4[sel].sum()))
            check(f"dim1M join seg {seg} equals GROUP BY amount folded by seg", (r7["results"][g, 0], r7["results"][g, 1]) == want)

        # the reference's closed-form table and known answers at the same row count
        cols = {"id": ops.Column.sequence(n, 1), "region": ops.Column.affine(n, 1, 0, cf.REGIONS),
                "amount": ops.Column.affine(n, 1, 0, cf.AMOUNT_RANGE)}
        try:
            e = cf.expected(n)
            s, mn, mx = ops.aggregate_global([cols["amount"]])
            check("closed form SUM/MIN/MAX(amount)", [s[0], mn[0], mx[0]] == e["sum_min_max_amount"])
            check("closed form COUNT amount > 9990", ops.scan_simple([cols["amount"]], [(0, ops.CMP_GT, cf.HIGH_AMOUNT)])[0] == e["count_amount_gt_9990"])
            check("closed form COUNT region = 7", ops.scan_simple([cols["region"]], [(0, ops.CMP_EQ, 7)])[0] == e["count_region_eq_7"])
            row = cf.needle_row(n)
            cnt, rows = ops.scan_simple([cols["id"]], [(0, ops.CMP_EQ, row + 1)], want_rows=True, max_rows=16)
            check("closed form id lookup", cnt == 1 and list(rows) == [row])
            mk, c, sm, _, _ = ops.group_dense(cols["region"], [ops.FUNC_COUNT, ops.FUNC_SUM], [None, cols["amount"]])
            want = np.array(e["group_region"], dtype=np.float64)
            check("closed form GROUP BY region", mk == 0 and np.array_equal(c.astype(np.float64), want[:, 1]) and np.array_equal(sm[:, 1].astype(np.float64), want[:, 2]))
            mk, c, sm, _, _ = ops.group_dense(cols["amount"], [ops.FUNC_COUNT, ops.FUNC_SUM], [None, cols["region"]])
            want = np.array(e["group_amount"], dtype=np.int64)
            check("closed form GROUP BY amount", mk == 0 and np.array_equal(c.astype(np.int64), want[:, 1]) and np.array_equal(sm[:, 1], want[:, 2]))
            regions_k = np.arange(50, dtype=np.uint32)
            r = ops.join_aggregate(cols["region"], [ops.FUNC_COUNT, ops.FUNC_SUM], [None, cols["amount"]], regions_k,
                                   dim_rows=np.nonzero(regions_k // 10 == 2)[0])
            check("closed form join regions zone 2", [r["results"][0, 0], r["results"][0, 1]] == [float(x) for x in e["join_zone2"]])
            products_k = np.arange(cf.AMOUNT_RANGE, dtype=np.uint32)
            category = (products_k % 20).astype(np.float64)
            r = ops.join_aggregate(cols["amount"], [ops.FUNC_COUNT], [None], products_k, group_values=[category])
            ok = r["groups"] == 20
            for g in range(r["groups"]):
                cat = int(category[int(r["dim_row"][g])])
                ok = ok and r["results"][g, 0] == sum(cf.amount_rows(n, a) for a in range(cat, cf.AMOUNT_RANGE, 20))
            check("closed form join products GROUP BY category", ok)
        finally:
            for c in cols.values():
                if c.buffer is not None:
                    c.buffer.close()
    except AssertionError as err:
        return f"failed: {err}", len(checks)
    except Exception as err:   # a malformed answer (a missing group, a short array) is a failed check too
        return f"failed: {type(err).__name__}: {err}", len(checks)
    return "ok", len(checks)


def measured_traffic(kernel, rows):
    """DRAM bytes per launch of the dominant kernel from the committed ncu summary (bytes per row, captured
    at 100M rows), scaled to `rows`; None when no capture covers the kernel."""
    if kernel != "aggregate_dense_native":
        return None
    path = os.path.join(os.path.dirname(os.path.abspath(__file__)), "profiles", "dense_traffic_100M.md")
    try:
        for line in open(path):
            if line.startswith("traffic_bytes_per_row_per_launch:"):
                return float(line.split(":")[1]) * rows
    except OSError:
        return None
    return None


def profile_entries(native):
    lib = native.load_cuda()
    import ctypes as C
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


def cpu_suite_seconds(rows, threads):
    """Seconds the oracle (CPU restatement of the reference's operators) takes for the suite over the first
    `rows` rows of the seed-0 table, on `threads` host threads (0 = all)."""
    import numpy as np
    import oracle
    from computeql_gb300 import workloads
    oracle.set_threads(threads)
    h = workloads.fact_numpy(rows, gen=oracle.splitmix_u32)
    ids = np.arange(rows, dtype=np.uint32)
    d50 = {"k": np.arange(50, dtype=np.uint32), "name_id": oracle.splitmix_u32(50, workloads.DIM50_SEED, 2, 0, 10)}
    d1m = {"k": np.arange(1_000_000, dtype=np.uint32), "seg": oracle.splitmix_u32(1_000_000, workloads.DIM1M_SEED, 1, 0, 20)}
    t0 = time.perf_counter()
    oracle.aggregate_global_cpu(h["amount"])
    oracle.scan_and([(h["flag"], 1, 2)], rows)
    oracle.group_cpu_reduce(h["region"], [h["amount"]], 64)
    oracle.group_cpu_reduce(h["amount"], [h["region"]], 16384)
    oracle.scan_and([(ids, 0, rows // 3)], rows, want_rows=True)
    keep = np.where(d50["name_id"] == 3, 0, 0xFFFFFFFF).astype(np.uint32)
    oracle.join_aggregate(h["region"], h["amount"], d50["k"], keep, 1)
    oracle.join_aggregate(h["amount"], h["amount"], d1m["k"], d1m["seg"], 20)
    dt = time.perf_counter() - t0
    cores = oracle.lib().orc_threads()
    oracle.set_threads(0)
    return dt, cores


def cpu_baseline(rows, threads=0, single_core_rows=None):
    """The oracle on a bounded sample: rows/s over the suite with all host threads, and on one core over a
    tenth of the sample."""
    dt, cores = cpu_suite_seconds(rows, threads)
    out = {"value": N_QUERIES * rows / dt, "unit": UNIT, "cores": cores, "kind": "port",
           "sample": f"the {N_QUERIES}-query suite on the first {rows} rows of the seed-0 table ({dt:.2f} s)"}
    if single_core_rows:
        dt1, _ = cpu_suite_seconds(single_core_rows, 1)
        out["single_core_value"] = N_QUERIES * single_core_rows / dt1
        out["single_core_sample"] = f"the same suite on the first {single_core_rows} rows, one thread ({dt1:.2f} s)"
    return out


def run_reference(args, rank, world):
    if rank != 0:
        return 0
    rows = args.cpu_rows
    samples = []
    for i in range(args.warmup + args.steps):
        r = cpu_baseline(rows)
        if i >= args.warmup:
            samples.append(r)
    value = statistics.median(s["value"] for s in samples)
    line = {"impl": "reference", "metric": METRIC, "value": value, "unit": UNIT, "n_gpus": args.gpus, "steps": args.steps,
            "warmup": args.warmup, "ms_per_step": N_QUERIES * rows / value * 1e3, "higher_is_better": True, "scaling": "weak",
            "vs_baseline": None, "dtype": "u32", "data": "synthetic (splitmix64 seed 0)",
            "config": {"workload": f"1B-row 4 x u32 table + dim50 + dim1M query suite (CPU sample of {rows} rows)", "rows": rows,
                       "queries": N_QUERIES},
            "cpu_baseline": {"value": value, "unit": UNIT, "cores": samples[0]["cores"], "kind": "port", "sample": samples[0]["sample"]},
            "e2e": {"value": value, "unit": UNIT, "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0}}
    print(json.dumps(line))
    return 0


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=10)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", default="ours", choices=["ours", "reference"])
    ap.add_argument("--rows", type=int, default=1_000_000_000)
    ap.add_argument("--cpu-rows", type=int, default=CPU_SAMPLE_ROWS)
    ap.add_argument("--no-e2e", action="store_true")
    ap.add_argument("--no-cpu", action="store_true")
    ap.add_argument("--no-extra", action="store_true", help="skip the batched and served configurations' figures")
    args = ap.parse_args()
    args.warmup = max(args.warmup, 3)

    rank = int(os.environ.get("RANK", "0"))
    world = int(os.environ.get("WORLD_SIZE", "1"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    if args.impl == "reference":
        return run_reference(args, rank, world)

    # one GPU per rank: replicas of the whole workload (weak scaling, no data-path collective)
    if world > 1:
        os.environ["CUDA_VISIBLE_DEVICES"] = str(local)
    dist = None
    if world > 1:
        import torch.distributed as dist
        dist.init_process_group("gloo")

    from computeql_gb300 import build, native, ops, workloads
    build.build()
    native.init()
    lib = native.load_cuda()

    t = workloads.fact_table(args.rows)
    import numpy as np
    key = np.random.default_rng(1234 + rank).integers(0, args.rows)
    dims = workloads.dim_tables()
    queries = make_queries(ops, t, key, dims)

    for _ in range(args.warmup):
        for _, _, q in queries:
            q()

    clocks = Clocks()
    clocks.start()
    if dist:
        dist.barrier()
    lib.cqlcuda_kernel_profile_reset()
    lib.cqlcuda_kernel_profile_enable(1)
    launches0 = lib.cqlcuda_kernel_launch_count()
    step_ms = []
    for _ in range(args.steps):
        lib.cqlcuda_timer_begin()
        for _, _, q in queries:
            q()
        step_ms.append(lib.cqlcuda_timer_end_ms())
    launches = lib.cqlcuda_kernel_launch_count() - launches0
    clk = clocks.stop()
    prof = profile_entries(native)

    # the same steps again, each query on its own: wall time, kernel time and its kernels (not in `value`)
    per_query = {name: [] for name, _, _ in queries}
    per_query_device = {name: [] for name, _, _ in queries}
    per_query_kernels = {name: {} for name, _, _ in queries}   # kernel -> [ns, launches]
    for _ in range(args.steps):
        for name, _, q in queries:
            p0 = profile_entries(native)
            t0 = time.perf_counter()
            q()
            per_query[name].append((time.perf_counter() - t0) * 1e3)
            p1 = profile_entries(native)
            per_query_device[name].append(sum(ns - p0.get(k, (0, 0))[0] for k, (ns, _) in p1.items()) / 1e6)
            for k, (ns, cnt) in p1.items():
                d_ns, d_cnt = ns - p0.get(k, (0, 0))[0], cnt - p0.get(k, (0, 0))[1]
                if d_cnt:
                    acc = per_query_kernels[name].setdefault(k, [0, 0])
                    acc[0] += d_ns
                    acc[1] += d_cnt
    lib.cqlcuda_kernel_profile_enable(0)

    total_ms = sum(step_ms)
    if dist:
        import torch
        tt = torch.tensor([total_ms], dtype=torch.float64)
        dist.all_reduce(tt, op=dist.ReduceOp.MAX)
        total_ms = float(tt.item())
    ms_per_step = total_ms / args.steps
    nq = len(queries)
    value = world * nq * args.rows / (ms_per_step / 1e3)
    # the point lookup is credited with the table's rows (as the reference's scale cases count them), though its
    # zone map keeps one 8192-row chunk of the id sequence; without it the suite's rows are the other six queries'
    value_without_lookup = world * (nq - 1) * args.rows / (ms_per_step / 1e3)

    peak, peak_kind = hbm_peak()
    # The dominant kernel (the most CUDA-event time over the suite) gives the roofline: its algorithmic
    # bytes are those of the queries it is the main kernel of (each query's bytes: the distinct columns
    # it reads x rows x 4 B), over its own event time in those queries.
    main_kernel = {name: max(kd, key=lambda k: kd[k][0]) for name, kd in per_query_kernels.items() if kd}
    totals = {}
    for kd in per_query_kernels.values():
        for k, (ns, _) in kd.items():
            totals[k] = totals.get(k, 0) + ns
    top = max(totals, key=totals.get) if totals else None
    roofline = None
    if top:
        served = [(name, nbytes) for name, nbytes, _ in queries if main_kernel.get(name) == top and nbytes > 0]
        ns = sum(per_query_kernels[name][top][0] for name, _ in served)
        cnt = sum(per_query_kernels[name][top][1] for name, _ in served)
        total_bytes = sum(nbytes for _, nbytes in served) * args.steps
        if ns and cnt:
            bytes_per_launch = total_bytes / cnt
            # the launch duration is the timed region's (CUDA events on the launching stream, over the timed
            # steps); the per-query pass above only says which queries the kernel serves and their bytes
            timed_ns, timed_cnt = prof.get(top, (ns, cnt))
            achieved = bytes_per_launch * timed_cnt / (timed_ns / 1e9) / 1e9
            roofline = {"kernel": top, "bound": "hbm", "achieved": achieved, "peak": peak, "peak_kind": peak_kind, "unit": "GB/s",
                        "frac": achieved / peak, "traffic": measured_traffic(top, args.rows), "bytes_per_launch": bytes_per_launch,
                        "per_unit": "4 B per row of each distinct column the query reads", "queries": [n for n, _ in served],
                        "avg_launch_ms": timed_ns / timed_cnt / 1e6, "launches": timed_cnt, "timed_region": True,
                        "traffic_source": "profiles/dense_traffic_100M.md (ncu DRAM bytes per launch, scaled by rows)"}
    qstats = {}
    for name, nbytes, _ in queries:
        ms = statistics.median(per_query[name])
        dms = statistics.median(per_query_device[name])
        qstats[name] = {"ms": ms, "rows_per_s": args.rows / (ms / 1e3), "GBps": nbytes / (ms / 1e3) / 1e9 if nbytes else None,
                        "hbm_frac": nbytes / (ms / 1e3) / 1e9 / peak if nbytes else None, "kernel_ms": dms,
                        "kernel_hbm_frac": nbytes / (dms / 1e3) / 1e9 / peak if dms > 0 and nbytes else None,
                        "main_kernel": main_kernel.get(name)}
    kernels = {k: {"ms_avg": ns / c / 1e6, "launches": c} for k, (ns, c) in prof.items()}

    parity, parity_checks_run = parity_checks(ops, t, queries, dims, key)

    e2e = None
    if not args.no_e2e:
        e2e = run_e2e(args, native, ops, t, queries, lib, dims)

    cpu = None
    if rank == 0 and not args.no_cpu:
        cpu = cpu_baseline(args.cpu_rows, single_core_rows=args.cpu_rows // 10)

    batched = served = None
    if rank == 0 and not args.no_extra and world == 1:
        batched = run_batched(native, ops, lib)
        served = run_served(ops, workloads, t, dims)

    if rank == 0:
        line = {"metric": METRIC, "value": value, "unit": UNIT, "n_gpus": world, "steps": args.steps, "warmup": args.warmup,
                "ms_per_step": ms_per_step, "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "u32",
                "data": "synthetic (splitmix64 seed 0, generated on the device)",
                "config": {"workload": "1B-row 4 x u32 table (id sequence, region, amount, flag) + dim50 + dim1M, warm in HBM: "
                                       f"{len(queries)}-query suite",
                           "rows": args.rows, "queries": [q[0] for q in queries], "l2": "inputs larger than L2 (4 GB columns)",
                           "parallelism": f"replicas x{world}"},
                "value_without_point_lookup": value_without_lookup,
                "parity": parity, "parity_checks": parity_checks_run,
                "gpu_launches": launches, "queries": qstats, "kernels": kernels, "roofline": roofline, "clocks": clk,
                "e2e": e2e, "cpu_baseline": cpu, "batched": batched, "served": served}
        print(json.dumps(line))
    if dist:
        dist.destroy_process_group()
    return 0


def run_batched(native, ops, lib):
    """The batched configuration, outside the suite's timed region: 100M rows of 4 u32 (uniform [0, 2^16)) and
    4 f64 (uniform [0, 1)) columns, 512 COUNT + SUM queries over 29 WHERE shapes drawn like the reference's
    per-query kernel benchmark. Wall times of one shared scan picked by the autotuner, of the queries one at a
    time through their own generated kernels, and of the persistent scan; the three paths' answers compared."""
    import numpy as np
    from computeql_gb300 import opbench
    rows = 100_000_000
    rng = np.random.default_rng(4)
    cols = {f"u{i}": ops.Column.splitmix(rows, 4, 8, i, 1 << 16) for i in range(4)}
    cols.update({f"d{i}": ops.Column.from_numpy(rng.random(rows)) for i in range(4)})
    qs = opbench._batch_queries(512, 29, 9)
    progs = [ops.Program(w, cols) for w, _ in qs]
    sums = [s for _, s in qs]
    auto = ops.CQLOPS_BATCH_AUTOTUNE
    for _ in range(8):                      # the autotuner's trial runs, one per candidate form, then its pick
        ops.batch_aggregate(progs, sums, auto)

    def timed(fn, reps):
        walls, out = [], None
        for _ in range(reps):
            t0 = time.perf_counter()
            out = fn()
            walls.append((time.perf_counter() - t0) * 1e3)
        return statistics.median(walls), out
    auto_ms, (c_auto, s_auto, _) = timed(lambda: ops.batch_aggregate(progs, sums, auto), 3)
    form = native.load_ops().cqlops_batch_last_form()
    # one generated kernel per (shape, summed column): 116 here, past the default cap of 64 loaded kernels, which
    # would evict and recompile them in turn; the cap is raised for this path, its kernels compiled first
    lib.cqlcuda_set_generated_kernel_cap(256)
    for p_, s_ in zip(progs, sums):
        ops.fused_aggregate(p_, [s_])
    one_ms, one = timed(lambda: [ops.fused_aggregate(p, [s]) for p, s in zip(progs, sums)], 1)
    lib.cqlcuda_set_generated_kernel_cap(64)
    c_one = np.array([r[0] for r in one], dtype=np.uint64)
    s_one = np.array([r[1][0] for r in one], dtype=np.float64)
    cat = ops.BatchCatalog()
    halves = [(progs[:384], sums[:384]), (progs[384:], sums[384:])]
    for p_, s_ in halves:
        cat.aggregate(p_, s_, 8)
    with ops.PersistentScan(cat, progs, rows_per_thread=8, idle_us=500_000) as ps:
        for p_, s_ in halves:
            ps.run(p_, s_)
        pers_ms, got = timed(lambda: [ps.run(p_, s_) for p_, s_ in halves], 3)
    c_pers = np.concatenate([g[0] for g in got])
    s_pers = np.concatenate([g[1] for g in got])
    rel = np.abs(s_auto - s_one) / np.maximum(np.abs(s_one), 1e-300)
    for c in cols.values():
        c.buffer.close()
    return {"workload": "100M rows x (4 u32 + 4 f64), 512 COUNT + SUM queries over 29 WHERE shapes", "unit": "ms per batch of 512",
            "shared_scan_autotuned_ms": auto_ms, "autotuned_form": {"rows_per_thread": form & 0xff, "block": 256 * max(1, (form >> 8) & 0xff)}
            if form & 0xff else {"form": "tile"},
            "one_at_a_time_ms": one_ms, "persistent_ms": pers_ms, "speedup_vs_one_at_a_time": one_ms / auto_ms,
            "parity": "ok" if (np.array_equal(c_auto, c_one) and np.array_equal(c_auto, c_pers) and float(rel.max()) <= 1e-12
                               and np.array_equal(s_auto.view(np.uint64), s_pers.view(np.uint64))) else "failed",
            "parity_checks": "counts equal across the three paths; shared-scan sums within 1e-12 of the per-query kernels' and equal "
                             "to the persistent scan's bit for bit"}


def run_served(ops, workloads, t, dims):
    """The served configuration's mix (computeql_gb300/servebench.py) over resident tables of 1M and 100M rows
    and the suite's own 1B-row table, 1 s at each offered rate, the plain one-query-at-a-time server against the
    served one."""
    import contextlib
    import io
    from computeql_gb300 import servebench
    tables = [{"region": f.region, "amount": f.amount, "flag": f.flag} for f in (workloads.fact_table(1_000_000, seed=1),
                                                                                 workloads.fact_table(100_000_000, seed=2))]
    tables.append({"region": t.region, "amount": t.amount, "flag": t.flag})
    d50, d1m = dims
    d1m = dict(d1m)
    d1m["seg_f64"] = d1m["seg"].astype("float64")
    out = {"workload": "60/25/15 filter-aggregate / group-by / join-sort templates over resident 1M, 100M and 1B-row tables, "
                       "Poisson arrivals, 160 GB admission budget, 1 s a rate", "slo_p99_ms": 50.0}
    # the plain server already falls behind at 5000 QPS; the served one is also offered 16000
    rates = {"plain": [2000.0, 5000.0], "served": [2000.0, 5000.0, 16000.0]}
    for mode in ("plain", "served"):
        with contextlib.redirect_stdout(io.StringIO()):
            lines, summary = servebench.run_mode(mode, tables, (d50, d1m), rates[mode], 1.0, 3, 50.0, 160 << 30)
        out[mode] = {"max_qps_within_slo": summary["max_qps_within_slo"],
                     "rates": [{k: r[k] for k in ("offered_qps", "completed_qps", "p50_ms", "p95_ms", "p99_ms", "failed")} for r in lines]}
    for tab in tables[:2]:
        for c in tab.values():
            c.buffer.close()
    return out


def _canon(x):
    """a query result as nested plain values, comparable with =="""
    import numpy as np
    if isinstance(x, dict):
        return {k: _canon(v) for k, v in x.items()}
    if isinstance(x, (list, tuple)):
        return [_canon(v) for v in x]
    if isinstance(x, np.ndarray):
        return x.tolist()
    return x


def run_e2e(args, native, ops, t, queries, lib, dims):
    """The suite from page-locked HOST buffers, every step: the fact columns region, amount and flag and
    the dimension tables' device columns uploaded, the seven queries run, their results read back. Uploads
    go through the backend's stream slots (the reference's GPU_Stream) and overlap the queries: the upload
    of the next column runs while the queries that need only the columns already on the device run on the
    main lane."""
    import ctypes as C
    n = args.rows
    d50, d1m = dims
    device = {"region": t.region, "amount": t.amount, "flag": t.flag, "dim1m_k": d1m["k_col"], "dim1m_seg": d1m["seg_col"],
              "dim50_k": d50["k_col"]}
    host, nbytes = {}, {}
    for name, col in device.items():
        # the host copy of the column: page-locked memory from the backend (on the GPU's host node)
        nbytes[name] = col.rows * 4
        h = lib.cqlcuda_host_alloc(nbytes[name])
        if not h:
            raise RuntimeError("e2e: cqlcuda_host_alloc failed: " + native.last_error())
        lib.cqlcuda_buffer_read(col.buffer.handle, C.c_void_p(h), nbytes[name])
        host[name] = h
    by_name = {name: q for name, _, q in queries}
    # columns in upload order, each slot with the queries that can run once it (and those before it) arrived
    plan = [(["amount", "dim1m_k", "dim1m_seg"], ["sum_min_max_amount", "join_dim1m_group_by_seg"]),
            (["region", "dim50_k"], ["group_by_region", "group_by_amount_10k", "join_dim50_filtered", "point_lookup_id"]),
            (["flag"], ["count_flag_lt_2"])]
    assert sorted(q for _, qs in plan for q in qs) == sorted(by_name)
    stream = lib.cqlcuda_stream_alloc(len(plan))
    if not stream:
        raise RuntimeError("e2e: cqlcuda_stream_alloc failed: " + native.last_error())

    def upload(slot):
        names = plan[slot][0]
        ok = lib.cqlcuda_stream_slot_begin(stream, slot, sum(nbytes[c] for c in names), 0)
        for c in names:
            ok = ok and lib.cqlcuda_stream_copy(stream, slot, device[c].buffer.handle, C.c_void_p(host[c]), nbytes[c])
        ok = ok and lib.cqlcuda_stream_submit(stream, slot)
        if not ok:
            raise RuntimeError("e2e upload failed: " + native.last_error())

    h2d = sum(nbytes.values())
    resident = {name: _canon(q()) for name, q in by_name.items()}
    times = []
    last = {}
    phases = {}      # per step: the wait for each slot's upload and each query, on the host clock

    def phase(name, t):
        if record:
            phases.setdefault(name, []).append((time.perf_counter() - t) * 1e3)
    for i in range(args.warmup + max(2, args.steps // 2)):
        record = i >= args.warmup
        t0 = time.perf_counter()
        upload(0)
        for slot, (_, names) in enumerate(plan):
            tw = time.perf_counter()
            if not lib.cqlcuda_stream_wait(stream, slot):
                raise RuntimeError("e2e upload failed: " + native.last_error())
            phase(f"wait_upload_{slot}", tw)
            if slot + 1 < len(plan):
                upload(slot + 1)
            for q in names:
                tq = time.perf_counter()
                last[q] = by_name[q]()
                phase(q, tq)
        dt = time.perf_counter() - t0
        if i >= args.warmup:
            times.append(dt)
    # the uploaded columns are the resident ones' bytes: every answer of the last step equals its resident run
    e2e_parity = "ok" if all(_canon(last[q]) == resident[q] for q in by_name) else \
        "failed: " + ", ".join(q for q in by_name if _canon(last[q]) != resident[q])
    lib.cqlcuda_stream_release(stream)
    # the uploads alone, one after another, for the link rate
    uploads = []
    stream = lib.cqlcuda_stream_alloc(1)
    for i in range(3):
        t0 = time.perf_counter()
        lib.cqlcuda_stream_slot_begin(stream, 0, h2d, 0)
        for names, _ in plan:
            for c in names:
                lib.cqlcuda_stream_copy(stream, 0, device[c].buffer.handle, C.c_void_p(host[c]), nbytes[c])
        lib.cqlcuda_stream_submit(stream, 0)
        lib.cqlcuda_stream_wait(stream, 0)
        uploads.append(time.perf_counter() - t0)
    lib.cqlcuda_stream_release(stream)
    for h in host.values():
        lib.cqlcuda_host_free(C.c_void_p(h))
    ms = statistics.median(times) * 1e3
    upload_ms = min(uploads) * 1e3
    # results read back per step: partials/counters/group arrays of the queries (a few hundred KB)
    d2h = 2048 * 3 * 8 + 8 + 50 * 4 * 8 + 10000 * 4 * 8 + 8 + 2 * 8 + 20 * 2 * 8
    return {"value": len(queries) * n / (ms / 1e3), "unit": UNIT, "ms_per_step": ms, "h2d_bytes_per_step": h2d,
            "d2h_bytes_per_step": d2h, "upload_ms": upload_ms, "h2d_GBps": h2d / (upload_ms / 1e3) / 1e9, "parity": e2e_parity,
            "phases_ms": {k: round(statistics.median(v), 3) for k, v in phases.items()}, "steps_ms": [round(x * 1e3, 2) for x in times],
            "overlap": "each column's upload overlaps the queries over the columns already uploaded"}

if __name__ == "__main__":
    sys.exit(main())
