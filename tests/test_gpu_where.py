"""Per-query kernels (NVRTC), the interpreter and the fused filter operators against the oracle.

Counts and row sets must match bit for bit; whole-number sums, minimums and maximums exactly;
f64 sums within 1e-12 relative of the exact (math.fsum) sum of the matching rows.
"""
import ctypes as C
import math

import numpy as np
import pytest

from tests.where_shapes import oracle_mask, random_shape, string_arrays

pytestmark = pytest.mark.gpu
F64_RTOL = 1e-12
N = 300_007


@pytest.fixture(scope="module")
def env(gpu):
    from computeql_gb300 import ops
    rng = np.random.default_rng(2024)
    arrays = {}
    for k in range(4):
        arrays[f"u{k}"] = rng.integers(0, 1 << 16, N).astype(np.uint32)
        arrays[f"d{k}"] = rng.random(N)
    arrays["i"] = rng.integers(-1000, 1000, N).astype(np.int32)
    arrays["f"] = (rng.standard_normal(N) * 10).astype(np.float32)
    arrays["region"] = rng.integers(0, 50, N).astype(np.uint32)
    arrays["status"] = rng.integers(0, 5, N).astype(np.uint32)
    words = ["alpha", "bravo", "charlie", "delta", "echo", "foxtrot", "golf", "hotel"]
    svals = [words[int(x)] + str(int(y)) for x, y in zip(rng.integers(0, 8, N), rng.integers(0, 5, N))]
    arrays["s"] = string_arrays(svals)
    cols = {k: ops.Column.from_numpy(v) for k, v in arrays.items() if not isinstance(v, tuple)}
    cols["s"] = ops.StringColumn(svals, dictionary=False)
    cols["sd"] = ops.StringColumn(svals, dictionary=True)
    arrays["sd"] = arrays["s"]
    return ops, arrays, cols, svals


def literal(col, rng):
    if col.startswith("u"):
        return int(rng.integers(0, 1 << 16))
    if col.startswith("d"):
        return round(float(rng.random()), 4)
    return 0


def check_scan(ops, program, arrays, strategy):
    mask = oracle_mask(program, arrays)
    cnt, rows, ran = ops.scan_filter(program, strategy, want_rows=True)
    assert cnt == int(mask.sum())
    assert np.array_equal(rows, np.nonzero(mask)[0].astype(np.uint32))
    return ran


@pytest.mark.parametrize("seed", range(40))
def test_random_shapes_generated_and_interpreter(env, seed):
    ops, arrays, cols, _ = env
    rng = np.random.default_rng(seed)
    names = ["u0", "u1", "u2", "u3", "d0", "d1", "d2", "d3"]
    where = random_shape(rng, names, literal)
    p = ops.Program(where, {k: cols[k] for k in names})
    assert check_scan(ops, p, arrays, ops.SCAN_GENERATED) == ops.SCAN_GENERATED
    if p.stack_depth() <= 8:
        assert check_scan(ops, p, arrays, ops.SCAN_INTERPRETER) == ops.SCAN_INTERPRETER
    ran = check_scan(ops, p, arrays, ops.SCAN_AUTO)
    assert ran in (ops.SCAN_SIMPLE, ops.SCAN_GENERATED)


@pytest.mark.parametrize("where", [
    "(< i -3.5)", "(>= i -1000)", "(= i 17)", "(!= i 17)", "(= i 17.5)", "(!= i 17.5)", "(< i 1e12)", "(> i -1e12)",
    "(< f 0.1)", "(<= f 0.1)", "(> f -2.5)", "(>= f 1e40)", "(= f 0.5)", "(!= f 0.1)", "(< f -1e300)",
    "(= u0 70000)", "(!= u0 -1)", "(> u0 65535.5)", "(<= u0 0)",
    "(or (= region 7) (and (> i 0) (< f 3)))", "(in region 1 5 9 49)", "(not_in region 0 1 2)", "(< region u0)",
    "(and (is_not_null d0) (> d0 0.5))", "(is_null d1)", "u0", "(> d3 1e-300)",
])
def test_edge_literals_match_the_double_comparison(env, where):
    ops, arrays, cols, _ = env
    p = ops.Program(where, {k: cols[k] for k in ("i", "f", "u0", "region", "d0", "d1", "d3")})
    check_scan(ops, p, arrays, ops.SCAN_GENERATED)
    if p.stack_depth() <= 8:
        check_scan(ops, p, arrays, ops.SCAN_INTERPRETER)


@pytest.mark.parametrize("where", ["(= s 'alpha3')", "(!= s 'echo1')", "(< s 'charlie')", "(>= s 'golf2')", "(contains s 'ho')",
                                   "(and (contains s 'a') (< u0 30000))", "(or (= s 'delta0') (= s 'delta4'))"])
def test_raw_string_predicates(env, where):
    ops, arrays, cols, _ = env
    p = ops.Program(where, {"s": cols["s"], "u0": cols["u0"]})
    check_scan(ops, p, arrays, ops.SCAN_GENERATED)
    check_scan(ops, p, arrays, ops.SCAN_INTERPRETER)


def test_dictionary_string_equality(env):
    ops, arrays, cols, svals = env
    for lit, expect in (("hotel2", sum(v == "hotel2" for v in svals)), ("nothere", 0)):
        p = ops.Program(f"(= sd '{lit}')", {"sd": cols["sd"], "u0": cols["u0"]})
        cnt, _, _ = ops.scan_filter(p, ops.SCAN_AUTO)
        assert cnt == expect
    # an absent literal folds to FALSE (and != to TRUE): the scan still runs over the table's rows
    p = ops.Program("(!= sd 'nothere')", {"sd": cols["sd"], "u0": cols["u0"]})
    assert ops.scan_filter(p, ops.SCAN_GENERATED)[0] == N
    p = ops.Program("(and (= sd 'bravo1') (< u0 40000))", {"sd": cols["sd"], "u0": cols["u0"]})
    check_scan(ops, p, arrays, ops.SCAN_GENERATED)


def test_deep_or_chain_runs_generated_not_interpreted(env):
    ops, arrays, cols, _ = env
    where = "(< u0 100)"
    for k in range(11):
        where = f"(or (= region {k}) {where})"
    # right-nested: every OR waits for the next one, depth 13
    nested = "(< u0 100)"
    for k in range(11):
        nested = f"(or {nested} (and (> u1 {k * 5000}) (< d0 {0.05 * k})))"
    for w in (where, nested):
        p = ops.Program(w, {"u0": cols["u0"], "u1": cols["u1"], "region": cols["region"], "d0": cols["d0"]})
        check_scan(ops, p, arrays, ops.SCAN_GENERATED)
    p = ops.Program(nested, {"u0": cols["u0"], "u1": cols["u1"], "d0": cols["d0"]})
    if p.stack_depth() > 8:
        with pytest.raises(ops.OpError, match="stack"):
            ops.scan_filter(p, ops.SCAN_INTERPRETER)


def test_literals_share_one_kernel(env):
    ops, arrays, cols, _ = env
    from computeql_gb300 import native
    lib = native.load_cuda()
    a, b = C.c_uint64(), C.c_uint64()
    ops.scan_filter(ops.Program("(or (< u0 100) (> d1 0.5))", {"u0": cols["u0"], "d1": cols["d1"]}), ops.SCAN_GENERATED)
    lib.cqlcuda_generated_kernel_stats(C.byref(a), None)
    for lit in (5, 700, 60000):
        p = ops.Program(f"(or (< u0 {lit}) (> d1 {lit / 70000}))", {"u0": cols["u0"], "d1": cols["d1"]})
        check_scan(ops, p, arrays, ops.SCAN_GENERATED)
    lib.cqlcuda_generated_kernel_stats(C.byref(b), None)
    assert b.value == a.value


def test_failed_compile_falls_back_to_the_interpreter(env):
    ops, arrays, cols, _ = env
    from computeql_gb300 import native
    lib = native.load_cuda()
    lib.cqlcuda_set_fail_compile_every(1)
    try:
        p = ops.Program("(or (> u2 123) (< d2 0.0123))", {"u2": cols["u2"], "d2": cols["d2"]})
        assert check_scan(ops, p, arrays, ops.SCAN_AUTO) == ops.SCAN_INTERPRETER
        with pytest.raises(ops.OpError):
            ops.scan_filter(p, ops.SCAN_GENERATED)
    finally:
        lib.cqlcuda_set_fail_compile_every(0)


@pytest.mark.parametrize("seed", range(10))
def test_fused_filter_aggregate(env, seed):
    ops, arrays, cols, _ = env
    rng = np.random.default_rng(100 + seed)
    names = ["u0", "u1", "u2", "u3", "d0", "d1", "d2", "d3"]
    where = random_shape(rng, names, literal)
    use = {k: cols[k] for k in names}
    use["i"] = cols["i"]
    use["f"] = cols["f"]
    p = ops.Program(where, use)
    mask = oracle_mask(p, arrays).astype(bool)
    cnt, s, mn, mx = ops.fused_aggregate(p, ["u1", "i", "d2", "f"])
    assert cnt == float(mask.sum())
    if mask.any():
        assert s[0] == float(arrays["u1"][mask].astype(np.int64).sum())
        assert (mn[0], mx[0]) == (float(arrays["u1"][mask].min()), float(arrays["u1"][mask].max()))
        assert s[1] == float(arrays["i"][mask].astype(np.int64).sum())
        assert (mn[1], mx[1]) == (float(arrays["i"][mask].min()), float(arrays["i"][mask].max()))
        exact = math.fsum(arrays["d2"][mask])
        assert abs(s[2] - exact) <= F64_RTOL * max(abs(exact), 1e-300)
        assert (mn[2], mx[2]) == (float(arrays["d2"][mask].min()), float(arrays["d2"][mask].max()))
        exact_f = math.fsum(arrays["f"][mask].astype(np.float64))
        assert abs(s[3] - exact_f) <= F64_RTOL * max(float(np.abs(arrays["f"][mask].astype(np.float64)).sum()), 1e-300)
        assert (mn[3], mx[3]) == (float(arrays["f"][mask].min()), float(arrays["f"][mask].max()))
    else:
        assert s[0] == 0.0 and mn[0] == 1.7976931348623157e308 and mx[0] == -1.7976931348623157e308


def test_fused_count_where_matches_scan(env):
    ops, arrays, cols, _ = env
    p = ops.Program("(< u0 1311)", {"u0": cols["u0"]})
    cnt, _, _, _ = ops.fused_aggregate(p, [])
    assert cnt == float((arrays["u0"] < 1311).sum())


@pytest.mark.parametrize("where", ["", "(< u0 20000)", "(or (> d0 0.9) (= region 3))"])
def test_fused_filter_group(env, where):
    ops, arrays, cols, svals = env
    use = {"u0": cols["u0"], "d0": cols["d0"], "region": cols["region"], "i": cols["i"], "sd": cols["sd"], "u1": cols["u1"],
           "status": cols["status"]}
    p = ops.Program(where, use)
    mask = oracle_mask(p, arrays).astype(bool) if where else np.ones(N, dtype=bool)
    # 5 x 40 groups x (2 + 4 x 2) words: inside the reference's 4096-word table
    res = ops.fused_group(p, ["status", "sd"], ["u1", "i"])
    codes = cols["sd"].codes
    ndict = int(codes.max()) + 1
    assert res["key_range"] == [5, ndict]
    g = arrays["status"].astype(np.int64) * ndict + codes
    for gi in range(res["groups"]):
        sel = mask & (g == gi)
        assert res["counts"][gi] == sel.sum()
        if sel.any():
            assert res["min_row"][gi] == np.nonzero(sel)[0][0]
            assert res["sums"][gi, 0] == arrays["u1"][sel].astype(np.int64).sum()
            assert res["sums"][gi, 1] == arrays["i"][sel].astype(np.int64).sum()
            assert res["mins"][gi, 0] == arrays["u1"][sel].min() and res["maxs"][gi, 0] == arrays["u1"][sel].max()
            assert res["mins"][gi, 1] == arrays["i"][sel].min() and res["maxs"][gi, 1] == arrays["i"][sel].max()


def test_fused_group_refuses_what_the_reference_refuses(env):
    ops, arrays, cols, _ = env
    p = ops.Program("(< u0 5)", {"u0": cols["u0"], "d0": cols["d0"], "u1": cols["u1"]})
    with pytest.raises(ops.OpError, match="16 KB"):
        ops.fused_group(p, ["u0"], ["u1"], max_groups=1 << 17)
    with pytest.raises(ops.OpError, match="U32/I32"):
        ops.fused_group(p, ["u0"], ["d0"])


@pytest.mark.parametrize("where", [
    "(< x 0.0)", "(<= x 0.0)", "(= x 0.0)", "(!= x 0.0)", "(> x -0.0)", "(>= x -0.0)", "(< x -1e308)", "(> x 1e308)",
    "(<= x -1e308)", "(>= x 1e308)", "(= x 2.5)", "(!= x 2.5)", "(< x 2.5)", "(> x -7.25)", "(and (> x -1.0) (< x 1.0))",
])
def test_f64_special_values(env, where):
    # -0.0, +-inf, NaN and literals at them: the generated kernels compare order keys, not doubles
    ops, _, _, _ = env
    rng = np.random.default_rng(17)
    x = rng.normal(size=50_003) * 3
    x[::11] = 0.0
    x[1::13] = -0.0
    x[2::17] = np.inf
    x[3::19] = -np.inf
    x[4::23] = np.nan
    x[5::29] = 2.5
    x[6::31] = -7.25
    x[7::37] = 1e308
    x[8::41] = -1e308
    arrays = {"x": x}
    p = ops.Program(where, {"x": ops.Column.from_numpy(x)})
    check_scan(ops, p, arrays, ops.SCAN_GENERATED)
    check_scan(ops, p, arrays, ops.SCAN_INTERPRETER)
