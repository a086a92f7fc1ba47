"""Served QPS and latency percentiles under open-loop Poisson arrivals: the served form against the plain
one-query-at-a-time path, at the same offered loads.

    python -m computeql_gb300.servebench [--sizes 1000000,100000000,1000000000] [--rates 50,200,1000,2000,5000]
                                         [--seconds S] [--workers W] [--mode both|served|plain] [--slo-ms MS]
                                         [--budget-gb 160]

The served configuration: a mix of the 10M/1B-row and wide-table configurations' query templates with fresh
literals over resident fact tables of 1M, 100M and 1B rows (region U[0,50), amount U[0,10000), flag U[0,100);
splitmix64, generated on the device), the dimension tables dim50 and dim1M resident too, and admission by
planned device footprint under a 160 GB budget. A request picks its table (1M 45 %, 100M 40 %, 1B 15 %)
and its template:

  filter/aggregate 60 %   count_flag      COUNT(*) WHERE flag < L
                          sum_region      SUM(amount) WHERE region = R
                          sum_mixed       SUM(amount) WHERE flag < L AND region >= A AND region < B
                          count_amount    COUNT(*) WHERE amount >= A AND amount < B
                          sum_or          SUM(amount) WHERE (region = R OR region = S) AND flag >= L
                          global          SUM/MIN/MAX(amount)
  group-by 25 %           by_region       SELECT region, COUNT(*), SUM(amount) GROUP BY region
                          by_flag         SELECT flag, COUNT(*), SUM(amount) GROUP BY flag
  join/sort 15 %          join_dim50      COUNT(*), SUM(amount) FROM fact JOIN dim50 ON region = k WHERE name_id = L
                          join_dim1m      seg, SUM(amount), COUNT(*) FROM fact JOIN dim1M ON amount = k GROUP BY seg
                          top_amount      SELECT id WHERE flag = L ORDER BY amount DESC LIMIT 100

A request's latency runs from its scheduled arrival (a late submit counts against the server) to the moment a
worker finished it. Two servers are measured:

  plain   one worker, no fusing: the reference's one-query-at-a-time serving (g_query_exec_mutex)
  served  `workers` workers on their own streams; filter/aggregate requests on a table fused into shared
          scans, identical group-bys merged; joins and sorts run as native call requests on the workers' lanes

One JSON line per (mode, rate), and a summary line per mode: the highest offered rate whose p99 stays within the
SLO while the server keeps up (completed rate >= 95 % of offered). Every request is built before the clock
starts (a server receives its queries parsed); the shapes are prepared (compiled) before it too.
"""
from __future__ import annotations

import argparse
import ctypes as C
import json
import time

import numpy as np

from . import build, native, ops, workloads

FILTER = ["count_flag", "sum_region", "sum_mixed", "count_amount", "sum_or"]
TEMPLATES = FILTER + ["global", "by_region", "by_flag", "join_dim50", "join_dim1m", "top_amount"]
WEIGHTS = [0.11] * 5 + [0.05, 0.125, 0.125, 0.05, 0.05, 0.05]
TABLE_WEIGHTS = [0.45, 0.40, 0.15]


def _where(kind, rng):
    if kind == "count_flag":
        return f"(< flag {int(rng.integers(1, 100))})", None
    if kind == "sum_region":
        return f"(= region {int(rng.integers(0, 50))})", "amount"
    if kind == "sum_mixed":
        a = int(rng.integers(0, 45))
        return f"(and (< flag {int(rng.integers(1, 100))}) (and (>= region {a}) (< region {a + int(rng.integers(1, 6))})))", "amount"
    if kind == "count_amount":
        a = int(rng.integers(0, 9000))
        return f"(and (>= amount {a}) (< amount {a + int(rng.integers(1, 1000))}))", None
    if kind == "sum_or":
        return (f"(and (or (= region {int(rng.integers(0, 50))}) (= region {int(rng.integers(0, 50))})) (>= flag {int(rng.integers(0, 100))}))",
                "amount")
    raise ValueError(kind)


def _plan(rate, seconds, seed, tables):
    rng = np.random.default_rng(seed)
    n = max(1, int(rng.poisson(rate * seconds)))
    gaps = rng.exponential(1.0 / rate, n)
    at = np.cumsum(gaps) - gaps[0]
    kinds = rng.choice(len(TEMPLATES), size=n, p=WEIGHTS)
    tw = np.array(TABLE_WEIGHTS[:tables], dtype=np.float64)
    which = rng.choice(tables, size=n, p=tw / tw.sum())
    return at, kinds, which, rng


def build_request(server, tab, kind, rng, dims):
    """one request of a template with fresh literals, not yet submitted"""
    table, cols = tab
    d50, d1m = dims
    name = TEMPLATES[kind]
    if name in FILTER:
        where, s = _where(name, rng)
        return server.filter_agg(table, table.program(where), s, submit=False)
    if name == "global":
        return server.agg_global(table, ["amount"], submit=False)
    if name in ("by_region", "by_flag"):
        return server.group_dense(table, name[3:], [ops.FUNC_COUNT, ops.FUNC_SUM], [None, "amount"], submit=False)
    if name == "join_dim50":
        kept = np.nonzero(d50["name_id"] == int(rng.integers(0, 10)))[0]
        return server.join(cols["region"], [ops.FUNC_COUNT, ops.FUNC_SUM], [None, cols["amount"]], d50["k"], dim_rows=kept,
                           dim_key_col=d50["k_col"], submit=False)
    if name == "join_dim1m":
        return server.join(cols["amount"], [ops.FUNC_SUM, ops.FUNC_COUNT], [cols["amount"], None], d1m["k"],
                           group_values=[d1m["seg_f64"]], dim_key_col=d1m["k_col"], dim_group_col=d1m["seg_col"], submit=False)
    if name == "top_amount":
        rows = cols["flag"].rows
        return server.sort([cols["flag"], cols["amount"]], [(0, ops.CMP_EQ, int(rng.integers(0, 100)))], 1, True, 100,
                           max(rows // 50, 1024), submit=False)
    raise ValueError(name)


def run_rate(server, tabs, dims, rate, seconds, seed):
    at, kinds, which, rng = _plan(rate, seconds, seed, len(tabs))
    reqs = [build_request(server, tabs[w], k, rng, dims) for k, w in zip(kinds, which)]
    lib = native.load_ops()
    handle = server.h
    ptrs = [C.byref(r.req) for r in reqs]
    t0 = time.monotonic_ns() + 20_000_000
    due = (t0 + at * 1e9).astype(np.int64).tolist()
    for i in range(len(reqs)):
        while True:
            wait = due[i] - time.monotonic_ns()
            if wait <= 0:
                break
            if wait > 300_000:
                time.sleep((wait - 200_000) / 1e9)
        lib.cqlserve_submit(handle, ptrs[i])
    for r in reqs:
        r.wait(0)
    done = np.array([r.req.done_ns for r in reqs], dtype=np.int64)
    ok = np.array([r.ok for r in reqs])
    lat_ms = (done - due) / 1e6
    span_s = (done.max() - t0) / 1e9
    fused = np.array([r.fused for r in reqs])
    fa = np.array([TEMPLATES[k] in FILTER for k in kinds])
    by_kind = {}
    for cat, names in (("filter_agg", FILTER + ["global"]), ("group_by", ["by_region", "by_flag"]),
                       ("join_sort", ["join_dim50", "join_dim1m", "top_amount"])):
        m = np.array([TEMPLATES[k] in names for k in kinds])
        if m.any():
            by_kind[cat] = {"requests": int(m.sum()), "p50_ms": float(np.percentile(lat_ms[m], 50)),
                            "p99_ms": float(np.percentile(lat_ms[m], 99))}
    errors = sorted({r.error for r in reqs if not r.ok})[:3]
    return {"offered_qps": rate, "requests": len(reqs), "failed": int((~ok).sum()), "errors": errors, "completed_qps": len(reqs) / span_s,
            "p50_ms": float(np.percentile(lat_ms, 50)), "p95_ms": float(np.percentile(lat_ms, 95)),
            "p99_ms": float(np.percentile(lat_ms, 99)), "max_ms": float(lat_ms.max()),
            "mean_fused": float(fused[fa].mean()) if fa.any() else 0.0, "by_category": by_kind}


def run_mode(mode, tables_cols, dims, rates, seconds, workers, slo_ms, budget):
    fuse = mode == "served"
    with ops.Server(workers=workers if fuse else 1, fuse=fuse, memory_budget=budget) as sv:
        tabs = []
        rng = np.random.default_rng(1)
        for cols in tables_cols:
            table = sv.add_table(cols)
            warm = [(k, *_where(k, rng)) for k in FILTER]
            sv.prepare(table, [table.program(w) for _, w, _ in warm], [s for _, _, s in warm])
            tabs.append((table, cols))
        # warm-up: every template on every table once (kernels compiled, pooled buffers sized)
        rs = [build_request(sv, tab, k, rng, dims) for tab in tabs for k in range(len(TEMPLATES))]
        for r in rs:
            sv.submit(r)
        for r in rs:
            r.wait(0)
            if not r.ok:
                raise ops.OpError(f"warm-up request failed: {r.error}")
        lines = []
        for i, rate in enumerate(rates):
            res = run_rate(sv, tabs, dims, rate, seconds, 100 + i)
            res.update({"mode": mode, "tables": [c["region"].rows for c in tables_cols], "workers": workers if fuse else 1,
                        "seconds": seconds, "memory_budget": budget})
            print(json.dumps(res), flush=True)
            lines.append(res)
        stats = sv.stats()
    good = [r["offered_qps"] for r in lines if r["p99_ms"] <= slo_ms and r["completed_qps"] >= 0.95 * r["offered_qps"] and not r["failed"]]
    summary = {"mode": mode, "summary": True, "slo_p99_ms": slo_ms, "max_qps_within_slo": max(good) if good else 0,
               "scans": stats["scans"], "fused_requests": stats["fused_requests"], "max_fused": stats["max_fused"],
               "merged_requests": stats["merged_requests"], "admission_waits": stats["admission_waits"],
               "peak_in_flight_bytes": stats["peak_in_flight_bytes"], "memory_budget": stats["memory_budget"]}
    print(json.dumps(summary), flush=True)
    return lines, summary


def main(argv=None):
    ap = argparse.ArgumentParser()
    ap.add_argument("--sizes", default="1000000,100000000,1000000000")
    ap.add_argument("--rates", default="50,200,1000,2000,5000")
    ap.add_argument("--seconds", type=float, default=2.0)
    ap.add_argument("--workers", type=int, default=3)
    ap.add_argument("--mode", default="both", choices=["both", "served", "plain"])
    ap.add_argument("--slo-ms", type=float, default=50.0)
    ap.add_argument("--budget-gb", type=float, default=160.0)
    args = ap.parse_args(argv)
    build.build()
    native.init()
    tables_cols = []
    for i, rows in enumerate(int(s) for s in args.sizes.split(",")):
        f = workloads.fact_table(rows, seed=i)
        tables_cols.append({"region": f.region, "amount": f.amount, "flag": f.flag})
    d50, d1m = workloads.dim_tables()
    d1m["seg_f64"] = d1m["seg"].astype(np.float64)
    rates = [float(r) for r in args.rates.split(",")]
    for mode in (["plain", "served"] if args.mode == "both" else [args.mode]):
        run_mode(mode, tables_cols, (d50, d1m), rates, args.seconds, args.workers, args.slo_ms, int(args.budget_gb * (1 << 30)))


if __name__ == "__main__":
    main()
