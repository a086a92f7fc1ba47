"""Writes the committed fixtures of tests/golden/.

closed_form_<n>.json - the answers of the reference's scale cases (src/tests/scale/bench_select_scale.c:97-160,
                       :1127-1170) at n rows of its closed-form table, from the formulas restated in
                       tests/closed_form.py.
c1_oracle.json       - the answers of the 10M-row configuration's queries on its seeded synthetic table
                       (computeql_gb300/workloads.py), computed by the oracle.

Run from the repository root: python tests/golden/make_golden.py
"""
import json
import os
import sys

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))
sys.path.insert(0, ROOT)

from tests import closed_form as cf  # noqa: E402


def write_closed_form(n):
    exp = cf.expected(n)
    exp.pop("group_amount")  # 10k rows of it: recomputed by the tests from the formula instead
    exp["rows"] = n
    with open(os.path.join(HERE, f"closed_form_{n}.json"), "w") as f:
        json.dump(exp, f, indent=1)


def write_c1():
    import numpy as np
    import oracle
    from computeql_gb300 import workloads
    n = 10_000_000
    t = workloads.fact_numpy(n, gen=oracle.splitmix_u32)
    s, mn, mx = oracle.aggregate_global_cpu(t["amount"])
    cnt, _ = oracle.scan_and([(t["flag"], 1, 2)], n)
    counts, sums, _, _ = oracle.group_dense(t["region"], 0, 50, [1, 0], [t["amount"], None])
    out = {
        "rows": n,
        "sum_min_max_amount": [s, mn, mx],
        "count_flag_lt_2": int(cnt),
        "group_region_sum_amount_count": [[g, int(sums[g, 0]), int(counts[g])] for g in range(50)],
        "first_rows": {k: [int(x) for x in t[k][:8]] for k in ("region", "amount", "flag")},
    }
    with open(os.path.join(HERE, "c1_oracle.json"), "w") as f:
        json.dump(out, f, indent=1)


if __name__ == "__main__":
    for n in (10001, 1000003):
        write_closed_form(n)
    write_c1()
