"""The wide-table configuration: nine queries over the 10M-row, 30-column event table, timed warm.

    python -m computeql_gb300.eventbench [--rows N] [--reps R]

The table (`workloads.event_numpy`) and its users table are resident in HBM before the clock starts. Each
query is one call of the operator that answers it, timed as the median wall time of `reps` calls after two
warm-up calls (results read back to host memory), with the kernel time of the same calls from CUDA events.
`reference_ms` is the reference's published time for the query on an RX 6700 XT (README.md:38-48), where
it publishes one.

  group_by_dict_string       SELECT s0, COUNT(*) GROUP BY s0 (200 dictionary values)
  group_by_status_f64        SELECT status, SUM(m0), SUM(m1), SUM(m2) GROUP BY status
  dict_string_eq_filter      SELECT rows WHERE s1 = <a dictionary value>
  group_by_region_5_aggs     SELECT region, COUNT(*), SUM(u0), MIN(u1), MAX(u2), AVG(u3) GROUP BY region
  three_predicate_filter     SELECT rows WHERE u4 >= A AND u4 < B AND m3 > X AND s2 = <value>
  join_users_by_segment      SELECT segment, COUNT(*), SUM(u5) FROM events JOIN users USING (user_id) GROUP BY segment
  group_by_user_id           SELECT user_id, COUNT(*), SUM(m0) GROUP BY user_id (1M groups)
  approx_distinct_session    SELECT APPROX_COUNT_DISTINCT(session) (4M distinct values)
  order_by_f64_filtered      SELECT rows WHERE region < 5 AND status = 1 ORDER BY m4 (200k rows, ties by row)
"""
from __future__ import annotations

import argparse
import json
import statistics
import time

import numpy as np

from . import build, native, ops, workloads

REFERENCE_MS = {"group_by_dict_string": 0.43, "group_by_status_f64": 0.79, "dict_string_eq_filter": 0.31,
                "group_by_region_5_aggs": 1.0, "three_predicate_filter": 1.1, "join_users_by_segment": 10.5,
                "group_by_user_id": 56.0, "approx_distinct_session": None, "order_by_f64_filtered": 9.5}

EQ_WORD, TRIPLE_WORD = 3, 0          # the dictionary values the string filters compare with
U4_LO, U4_HI, M3_GT = 100_000, 600_000, 20.0


def programs(cols, words):
    """The two WHERE programs of the suite: the dictionary equality and the three-predicate filter."""
    return {"eq": ops.Program(f"(= s1 '{words[EQ_WORD]}')", {"s1": cols["s1"]}),
            "triple": ops.Program(f"(and (and (>= u4 {U4_LO}) (< u4 {U4_HI})) (and (> m3 {M3_GT!r}) (= s2 '{words[TRIPLE_WORD]}')))",
                                  {"u4": cols["u4"], "m3": cols["m3"], "s2": cols["s2"]})}


def queries(cols, users, words):
    """The suite as (name, callable) over the resident columns; each callable returns its result."""
    seg = users["segment"].astype(np.float64)
    progs = programs(cols, words)
    program_eq, program_triple = progs["eq"], progs["triple"]
    sort_filter = [(0, ops.CMP_LT, 5), (1, ops.CMP_EQ, 1)]

    def order_by_filtered():
        _, rows = ops.scan_simple([cols["region"], cols["status"]], sort_filter, want_rows=True)
        sel = ops.DeviceBuffer(max(rows.nbytes, 4), rows)
        return rows, ops.sort_rows([cols["m4"]], selection=sel, count=len(rows))

    return [
        ("group_by_dict_string", lambda: ops.group_dense(cols["s0"], [ops.FUNC_COUNT], [None])),
        ("group_by_status_f64", lambda: ops.group_hash([cols["status"]], [ops.FUNC_SUM] * 3, [cols["m0"], cols["m1"], cols["m2"]],
                                                       group_hint=5)),
        ("dict_string_eq_filter", lambda: ops.scan_filter(program_eq, want_rows=True)),
        ("group_by_region_5_aggs", lambda: ops.group_dense(cols["region"], [ops.FUNC_COUNT, ops.FUNC_SUM, ops.FUNC_MIN, ops.FUNC_MAX, ops.FUNC_AVG],
                                                           [None, cols["u0"], cols["u1"], cols["u2"], cols["u3"]])),
        ("three_predicate_filter", lambda: ops.scan_filter(program_triple, want_rows=True)),
        ("join_users_by_segment", lambda: ops.join_aggregate(cols["user_id"], [ops.FUNC_COUNT, ops.FUNC_SUM], [None, cols["u5"]],
                                                             users["user_id"], group_values=[seg])),
        ("group_by_user_id", lambda: ops.group_hash([cols["user_id"]], [ops.FUNC_COUNT, ops.FUNC_SUM], [None, cols["m0"]],
                                                    group_hint=1_000_000)),
        ("approx_distinct_session", lambda: ops.group_hash([], [ops.FUNC_ACD], [cols["session"]])),
        ("order_by_f64_filtered", order_by_filtered),
    ]


def _profile_ms(lib):
    import ctypes as C
    total, i = 0, 0
    while True:
        name, ns, cnt = C.c_char_p(), C.c_uint64(), C.c_uint64()
        if not lib.cqlcuda_kernel_profile_entry(i, C.byref(name), C.byref(ns), C.byref(cnt)):
            return total / 1e6
        total += ns.value
        i += 1


def main(argv=None):
    ap = argparse.ArgumentParser()
    ap.add_argument("--rows", type=int, default=10_000_000)
    ap.add_argument("--reps", type=int, default=10)
    args = ap.parse_args(argv)
    build.build()
    native.init()
    t0 = time.perf_counter()
    cols, users, _, words = workloads.event_table(args.rows)
    gen_s = time.perf_counter() - t0
    lib = native.load_cuda()
    for name, fn in queries(cols, users, words):
        fn()
        fn()
        lib.cqlcuda_kernel_profile_reset()
        lib.cqlcuda_kernel_profile_enable(1)
        walls = []
        for _ in range(args.reps):
            t = time.perf_counter()
            fn()
            walls.append((time.perf_counter() - t) * 1e3)
        lib.cqlcuda_kernel_profile_enable(0)
        kernel_ms = _profile_ms(lib) / args.reps
        wall = statistics.median(walls)
        ref = REFERENCE_MS[name]
        print(json.dumps({"query": name, "rows": args.rows, "wall_ms": round(wall, 4), "kernel_ms": round(kernel_ms, 4),
                          "reference_ms": ref, "reference_over_ours": round(ref / wall, 1) if ref else None}), flush=True)
    print(json.dumps({"summary": True, "rows": args.rows, "table_generation_s": round(gen_s, 1)}), flush=True)


if __name__ == "__main__":
    main()
