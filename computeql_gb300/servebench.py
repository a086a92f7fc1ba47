"""Served QPS and latency percentiles under Poisson arrivals, one query at a time against the server.

    python -m computeql_gb300.servebench [--rows N] [--rates 200,1000,...] [--seconds S] [--workers W]
                                         [--mode both|served|plain] [--slo-ms MS]

The table is the fact table of the 1B-row configuration (region U[0,50), amount U[0,10000),
flag U[0,100); splitmix64 seed 0, generated on the device and resident in HBM). Requests are drawn from
query templates with fresh literals each time, in the C1/C2 query families:

  count_flag     COUNT(*) WHERE flag < L                                      (filter/aggregate)
  sum_region     SUM(amount) WHERE region = R                                 (filter/aggregate)
  sum_mixed      SUM(amount) WHERE flag < L AND region >= A AND region < B   (filter/aggregate)
  count_amount   COUNT(*) WHERE amount >= A AND amount < B                    (filter/aggregate)
  sum_or         SUM(amount) WHERE (region = R OR region = S) AND flag >= L  (filter/aggregate)
  global         SUM/MIN/MAX(amount)                                          (whole column)
  by_region      SELECT region, COUNT(*), SUM(amount) GROUP BY region         (dense group-by)

in the proportions 18/18/18/17/17/6/6 %. Arrival times are a Poisson process at each offered rate for
`seconds`; a request's latency runs from its scheduled arrival (so a late submit counts against the
server) to the moment a worker finished it. Two servers are measured:

  plain   one worker, no fusing: the reference's one-query-at-a-time serving (g_query_exec_mutex)
  served  `workers` workers on their own streams, filter/aggregate requests fused into shared scans

One JSON line per (mode, rate) and a summary line per mode with the highest offered rate whose p99 stays
within the SLO while the server keeps up (completed rate >= 95% of offered). Every request is built before
the clock starts (a server receives its queries parsed; the timed loop only waits for each arrival and
queues it); the templates' shapes are prepared (compiled) before it too.
"""
from __future__ import annotations

import argparse
import ctypes as C
import json
import time

import numpy as np

from . import build, native, ops, workloads

TEMPLATES = ["count_flag", "sum_region", "sum_mixed", "count_amount", "sum_or", "global", "by_region"]
WEIGHTS = [0.18, 0.18, 0.18, 0.17, 0.17, 0.06, 0.06]


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


def _plan(rate, seconds, seed):
    rng = np.random.default_rng(seed)
    n = max(1, int(rng.poisson(rate * seconds)))
    gaps = rng.exponential(1.0 / rate, n)
    at = np.cumsum(gaps) - gaps[0]
    kinds = rng.choice(len(TEMPLATES), size=n, p=WEIGHTS)
    return at, kinds, rng


def _table(rows):
    f = workloads.fact_table(rows)
    return {"region": f.region, "amount": f.amount, "flag": f.flag}


def run_rate(server, table, rate, seconds, seed):
    at, kinds, rng = _plan(rate, seconds, seed)
    # every request built before the clock starts (a server receives its queries parsed): the timed loop
    # only waits for each arrival and queues it
    reqs = []
    for k in kinds:
        name = TEMPLATES[k]
        if name == "global":
            reqs.append(server.agg_global(table, ["amount"], submit=False))
        elif name == "by_region":
            reqs.append(server.group_dense(table, "region", [ops.FUNC_COUNT, ops.FUNC_SUM], [None, "amount"], submit=False))
        else:
            where, s = _where(name, rng)
            reqs.append(server.filter_agg(table, table.program(where), s, submit=False))
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
    fa = np.array([k < 5 for k in kinds])
    return {"offered_qps": rate, "requests": len(reqs), "failed": int((~ok).sum()), "completed_qps": len(reqs) / span_s,
            "p50_ms": float(np.percentile(lat_ms, 50)), "p95_ms": float(np.percentile(lat_ms, 95)),
            "p99_ms": float(np.percentile(lat_ms, 99)), "max_ms": float(lat_ms.max()),
            "mean_fused": float(fused[fa].mean()) if fa.any() else 0.0}


def run_mode(mode, cols, rates, seconds, workers, slo_ms, rows):
    fuse = mode == "served"
    with ops.Server(workers=workers if fuse else 1, fuse=fuse) as sv:
        table = sv.add_table(cols)
        rng = np.random.default_rng(1)
        warm = [(TEMPLATES[k], *_where(TEMPLATES[k], rng)) for k in range(5)]
        sv.prepare(table, [table.program(w) for _, w, _ in warm], [s for _, _, s in warm])
        # warm-up: every template once, the per-query kernels compiled
        rs = [sv.filter_agg(table, table.program(w), s) for _, w, s in warm]
        rs += [sv.agg_global(table, ["amount"]), sv.group_dense(table, "region", [ops.FUNC_COUNT, ops.FUNC_SUM], [None, "amount"])]
        for r in rs:
            r.wait(0)
            if not r.ok:
                raise ops.OpError(f"warm-up request failed: {r.error}")
        lines = []
        for i, rate in enumerate(rates):
            res = run_rate(sv, table, rate, seconds, 100 + i)
            res.update({"mode": mode, "rows": rows, "workers": workers if fuse else 1, "seconds": seconds})
            print(json.dumps(res), flush=True)
            lines.append(res)
        stats = sv.stats()
    good = [r["offered_qps"] for r in lines if r["p99_ms"] <= slo_ms and r["completed_qps"] >= 0.95 * r["offered_qps"] and not r["failed"]]
    summary = {"mode": mode, "summary": True, "slo_p99_ms": slo_ms, "max_qps_within_slo": max(good) if good else 0,
               "scans": stats["scans"], "fused_requests": stats["fused_requests"], "max_fused": stats["max_fused"],
               "peak_in_flight_bytes": stats["peak_in_flight_bytes"]}
    print(json.dumps(summary), flush=True)
    return lines, summary


def main(argv=None):
    ap = argparse.ArgumentParser()
    ap.add_argument("--rows", type=int, default=1_000_000_000)
    ap.add_argument("--rates", default="100,500,1000,2000,5000")
    ap.add_argument("--seconds", type=float, default=2.0)
    ap.add_argument("--workers", type=int, default=3)
    ap.add_argument("--mode", default="both", choices=["both", "served", "plain"])
    ap.add_argument("--slo-ms", type=float, default=50.0)
    args = ap.parse_args(argv)
    build.build()
    native.init()
    cols = _table(args.rows)
    rates = [float(r) for r in args.rates.split(",")]
    for mode in (["plain", "served"] if args.mode == "both" else [args.mode]):
        run_mode(mode, cols, rates, args.seconds, args.workers, args.slo_ms, args.rows)


if __name__ == "__main__":
    main()
