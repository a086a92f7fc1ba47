"""The oracle against the reference's own known answers (CPU only).

The closed-form table and expected answers are those of src/tests/scale/bench_select_scale.c
(restated in tests/closed_form.py); the committed fixtures in tests/golden/ hold the same answers
for fixed sizes, made by tests/golden/make_golden.py.
"""
import json
import os

import numpy as np
import pytest

import oracle
from tests import closed_form as cf

GOLDEN = os.path.join(os.path.dirname(__file__), "golden")
SIZES = [1, 2, 7, 49, 50, 51, 9999, 10000, 10001, 123457, 1000003]


def oracle_answers(n):
    idc, region, amount, needle = oracle.closed_form(n)
    s_cpu = oracle.aggregate_global_cpu(amount)
    s_gpu = oracle.aggregate_global_gpu_order(amount) if n <= 200000 else s_cpu
    high, _ = oracle.scan_and([(amount, 3, cf.HIGH_AMOUNT)], n)
    reg7, _ = oracle.scan_and([(region, 0, 7)], n)
    idr, _ = oracle.scan_and([(idc, 3, 1000), (idc, 2, 900000000)], n)
    counts, sums, _, _ = oracle.group_dense(region, 0, 50, [0, 1], [None, amount])
    gr = [[g, int(counts[g]), float(sums[g, 1])] for g in range(50) if counts[g] > 0]
    acount, asums, _, _ = oracle.group_dense(amount, 0, 10000, [0, 1], [None, region])
    ga = [[a, int(acount[a]), int(asums[a, 1])] for a in range(10000) if acount[a] > 0]
    zc, zrows = oracle.scan_and([(region, 4, 20), (region, 2, 29)], n, want_rows=True)
    zsum = float(amount[zrows].astype(np.float64).sum()) if zc else 0.0
    return {
        "sum_min_max_amount": list(s_cpu),
        "sum_min_max_amount_gpu_order": list(s_gpu),
        "count_amount_gt_9990": int(high),
        "count_region_eq_7": int(reg7),
        "count_id_range": int(idr),
        "group_region": gr,
        "group_amount": ga,
        "join_zone2": [int(zc), zsum],
    }


@pytest.mark.parametrize("n", SIZES)
def test_oracle_matches_closed_form(n):
    exp = cf.expected(n)
    got = oracle_answers(n)
    assert got["sum_min_max_amount"] == exp["sum_min_max_amount"]
    assert got["sum_min_max_amount_gpu_order"] == exp["sum_min_max_amount"]
    assert got["count_amount_gt_9990"] == exp["count_amount_gt_9990"]
    assert got["count_region_eq_7"] == exp["count_region_eq_7"]
    assert got["count_id_range"] == exp["count_id_range"]
    assert got["group_region"] == exp["group_region"]
    assert got["group_amount"] == exp["group_amount"]
    assert got["join_zone2"] == list(exp["join_zone2"])


@pytest.mark.parametrize("name", sorted(f for f in os.listdir(GOLDEN) if f.startswith("closed_form_")))
def test_oracle_matches_committed_fixture(name):
    with open(os.path.join(GOLDEN, name)) as f:
        fx = json.load(f)
    n = fx["rows"]
    got = oracle_answers(n)
    for k in ("sum_min_max_amount", "count_amount_gt_9990", "count_region_eq_7", "count_id_range", "group_region", "join_zone2"):
        assert got[k] == fx[k], k


def test_splitmix_matches_reference_stream():
    # bench_rng_next (src/tests/bench_common.h:30-37) with state 0: the first outputs of splitmix64
    expected = [0xE220A8397B1DCDAF, 0x6E789E6AA1B965F4, 0x06C45D188009454F]
    assert [oracle.lib().orc_splitmix_draw(0, k) for k in range(3)] == expected


def test_cpu_group_reduce_agrees_with_dense():
    n = 200000
    key = oracle.splitmix_u32(n, 5, 2, 0, 1000)
    arg = oracle.splitmix_u32(n, 5, 2, 1, 100000)
    keys, counts, sums, mins, maxs = oracle.group_cpu_reduce(key, [arg], 2000)
    dcount, dsum, dmin, dmax = oracle.group_dense(key, 0, 1000, [1, 3, 4], [arg, arg, arg])
    for k, c, s, lo, hi in zip(keys, counts, sums[:, 0], mins[:, 0], maxs[:, 0]):
        assert dcount[k] == c
        assert dsum[k, 0] == s
        assert dmin[k, 1] == lo and dmax[k, 2] == hi
