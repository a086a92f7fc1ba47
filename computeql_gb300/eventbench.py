"""The wide-table configuration: nine queries over the 10M-row, 30-column event table, timed warm.

    python -m computeql_gb300.eventbench [--rows N] [--reps R]

The table (`workloads.event_numpy`) and its users table are resident in HBM before the clock starts. Each
query is one call of the operator that answers it, timed as the median wall time of `reps` calls after two
warm-up calls (results read back to host memory), with the kernel time of the same calls from CUDA events.
The queries take the forms of the reference's wide-table benchmark (src/tests/scale/bench_query_xlarge.c:
492-567) over this table's columns; `reference_ms` is the reference's published time for that query on an
RX 6700 XT (README.md:38-48), where it publishes one.

  group_by_dict_string       SELECT s0, COUNT(*), SUM(u0) GROUP BY s0 (200 dictionary values)
  group_by_status_f64        SELECT status, SUM(m0), AVG(m1), MIN(m1), MAX(m1) GROUP BY status
  dict_string_eq_filter      SELECT COUNT(*) WHERE s1 = <a dictionary value>
  group_by_region_5_aggs     SELECT region, COUNT(*), SUM(u0), AVG(m0), MIN(m1), MAX(m1) GROUP BY region
  three_predicate_filter     SELECT COUNT(*), SUM(u5) WHERE region = 7 AND s2 = <value> AND u4 >= A AND u4 <= B
  join_users_by_segment      SELECT segment, COUNT(*), SUM(u5) FROM events JOIN users USING (user_id) GROUP BY segment
  group_by_user_id           SELECT user_id, COUNT(*), SUM(u0) GROUP BY user_id (1M groups)
  distinct_sessions          SELECT COUNT(*) FROM (SELECT session GROUP BY session) (4M values)
  sort_200k                  SELECT rows WHERE region = 3 ORDER BY m4 (200k rows, ties by row; the filter's rows
                             stay on the device for the sort)

and four more of that benchmark's forms, for which the reference publishes no time:

  wide_projection_1pct       SELECT * WHERE u1 > 1038090 (1 %): the rows and all 28 stored columns' values
  window_top3_per_region     SELECT COUNT(*) FROM (SELECT ROW_NUMBER() OVER (PARTITION BY region ORDER BY u2 DESC)
                             AS rn WHERE u0 > 943718) WHERE rn <= 3 (1M rows ranked)
  having_1m_groups           SELECT user_id, SUM(u0) GROUP BY user_id HAVING SUM(u0) > 8000000
  eight_measures_by_region   SELECT region, SUM(m0), ..., SUM(m7) GROUP BY region
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
                "group_by_user_id": 56.0, "distinct_sessions": None, "sort_200k": 9.5, "wide_projection_1pct": None,
                "window_top3_per_region": None, "having_1m_groups": None, "eight_measures_by_region": None}

EQ_WORD, TRIPLE_WORD = 3, 0          # the dictionary values the string filters compare with
TRIPLE_REGION, U4_LO, U4_HI = 7, 100_000, 900_000
SORT_REGION = 3
WIDE_U1_GT, WINDOW_U0_GT, HAVING_SUM_GT = 1_038_090, 943_718, 8_000_000
STORED = workloads.EVENT_U32 + workloads.EVENT_I64 + workloads.EVENT_F64 + ["user_id", "region", "status"] + workloads.EVENT_DICT + ["session"]


def programs(cols, words):
    """The two WHERE programs of the suite: the dictionary equality and the three-predicate filter."""
    return {"eq": ops.Program(f"(= s1 '{words[EQ_WORD]}')", {"s1": cols["s1"]}),
            "triple": ops.Program(f"(and (and (= region {TRIPLE_REGION}) (= s2 '{words[TRIPLE_WORD]}')) (and (>= u4 {U4_LO}) (<= u4 {U4_HI})))",
                                  {"region": cols["region"], "s2": cols["s2"], "u4": cols["u4"], "u5": cols["u5"]})}


def queries(cols, users, words):
    """The suite as (name, callable) over the resident columns; each callable returns its result."""
    seg = users["segment"].astype(np.float64)
    progs = programs(cols, words)
    program_eq, program_triple = progs["eq"], progs["triple"]
    F = ops

    stored = [cols[c] for c in STORED]
    # a filter's rows stay on the device for the operator after it (gather, sort, window), in a selection buffer
    # kept between calls as an engine keeps its scratch
    selection = ops.DeviceBuffer(cols["u0"].rows * 4)

    row_numbers = ops.Column.sequence(cols["u1"].rows)

    def wide_projection():
        # the filter's rows stay on the device; the row numbers come back with the values (a sequence column)
        n = ops.scan_select([cols["u1"]], [(0, ops.CMP_GT, WIDE_U1_GT)], selection)
        values = ops.gather_rows(stored + [row_numbers], selection=selection, count=n)
        return values[-1], values[:-1]

    window_out = {}

    def window_top3():
        n = ops.scan_select([cols["u0"]], [(0, ops.CMP_GT, WINDOW_U0_GT)], selection)
        w = ops.window_rank([cols["region"], cols["u2"]], desc=[0, 1], partitions=1, selection=selection, count=n,
                            want=("row_number",), out=window_out)
        return int(np.count_nonzero(w["row_number"] <= 3))

    # each hash group-by of many groups writes into its own result area, kept between calls as an engine keeps
    # its result buffers (fresh arrays would cost their page faults in every call)
    rows = cols["user_id"].rows
    out_users = ops.HashOutputs(min(rows, 2_000_000), 2)
    out_sessions = ops.HashOutputs(min(rows, 8_000_000), 1)
    out_having = ops.HashOutputs(min(rows, 2_000_000), 1)

    def having_1m():
        r = ops.group_hash([cols["user_id"]], [F.FUNC_SUM], [cols["u0"]], group_hint=1_000_000, out=out_having)
        keep = ops.having("v0 > lit[0]", [r["results"][:, 0]], [HAVING_SUM_GT])
        return r, keep

    def sort_200k():
        n = ops.scan_select([cols["region"]], [(0, ops.CMP_EQ, SORT_REGION)], selection)
        return ops.sort_rows([cols["m4"]], selection=selection, count=n)

    return [
        ("group_by_dict_string", lambda: ops.group_dense(cols["s0"], [F.FUNC_COUNT, F.FUNC_SUM], [None, cols["u0"]])),
        ("group_by_status_f64", lambda: ops.group_hash([cols["status"]], [F.FUNC_SUM, F.FUNC_AVG, F.FUNC_MIN, F.FUNC_MAX],
                                                       [cols["m0"], cols["m1"], cols["m1"], cols["m1"]], group_hint=5)),
        ("dict_string_eq_filter", lambda: ops.scan_filter(program_eq)),
        ("group_by_region_5_aggs", lambda: ops.group_hash([cols["region"]], [F.FUNC_COUNT, F.FUNC_SUM, F.FUNC_AVG, F.FUNC_MIN, F.FUNC_MAX],
                                                          [None, cols["u0"], cols["m0"], cols["m1"], cols["m1"]], group_hint=50)),
        ("three_predicate_filter", lambda: ops.fused_aggregate(program_triple, ["u5"])),
        ("join_users_by_segment", lambda: ops.join_aggregate(cols["user_id"], [F.FUNC_COUNT, F.FUNC_SUM], [None, cols["u5"]],
                                                             users["user_id"], group_values=[seg], dim_key_col=users.get("user_id_col"),
                                                             dim_group_col=users.get("segment_col"))),
        ("group_by_user_id", lambda: ops.group_hash([cols["user_id"]], [F.FUNC_COUNT, F.FUNC_SUM], [None, cols["u0"]],
                                                    group_hint=1_000_000, out=out_users)),
        ("distinct_sessions", lambda: ops.group_hash([cols["session"]], [F.FUNC_COUNT], [None], group_hint=4_000_000, out=out_sessions)),
        ("sort_200k", sort_200k),
        ("wide_projection_1pct", wide_projection),
        ("window_top3_per_region", window_top3),
        ("having_1m_groups", having_1m),
        ("eight_measures_by_region", lambda: ops.group_hash([cols["region"]], [F.FUNC_SUM] * 8, [cols[m] for m in workloads.EVENT_F64],
                                                            group_hint=50)),
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
