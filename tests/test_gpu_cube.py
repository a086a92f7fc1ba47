"""The cube form of the batched shared scan: queries whose WHERE reads only small-range whole-number
columns answered from one dense table of the rows (counts and exact fixed-point sums per combination of
those columns' values).

Every query must give what the oracle gives: its count bit for bit, its SUM within 1e-12 of math.fsum
of the matching rows, and the same integers as the scan answers (the same query in a batch that the cube
cannot take). The cube kernels must actually run (their launches are in the kernel profile), and a column
whose values leave its stated range must send its queries back to the scan with the right answers.
"""
import ctypes as C
import math

import numpy as np
import pytest

from tests.where_shapes import oracle_mask

pytestmark = pytest.mark.gpu

ROWS = 2_000_003


@pytest.fixture(scope="module")
def env(gpu):
    from computeql_gb300 import ops
    rng = np.random.default_rng(31)
    arrays = {
        "region": rng.integers(0, 50, ROWS).astype(np.uint32),
        "flag": rng.integers(0, 100, ROWS).astype(np.uint32),
        "status": rng.integers(-3, 6, ROWS).astype(np.int32),
        "amount": rng.integers(0, 10000, ROWS).astype(np.uint32),
        "v": rng.lognormal(3.0, 1.0, ROWS),
    }
    cols = {n: ops.Column.from_numpy(a) for n, a in arrays.items()}
    return ops, arrays, cols


def _profile(lib):
    out = {}
    i = 0
    while True:
        name, ns, cnt = C.c_char_p(), C.c_uint64(), C.c_uint64()
        if not lib.cqlcuda_kernel_profile_entry(i, C.byref(name), C.byref(ns), C.byref(cnt)):
            break
        if cnt.value:
            out[name.value.decode()] = cnt.value
        i += 1
    return out


def _run(ops, progs, sums, rpt=8):
    from computeql_gb300 import native
    lib = native.load_cuda()
    lib.cqlcuda_kernel_profile_reset()
    lib.cqlcuda_kernel_profile_enable(1)
    counts, vals, _ = ops.batch_aggregate(progs, sums, rpt)
    lib.cqlcuda_kernel_profile_enable(0)
    return counts, vals, _profile(lib)


def _queries(rng, n):
    out = []
    for q in range(n):
        kind = q % 7
        if kind == 0:
            out.append((f"(< flag {int(rng.integers(1, 100))})", None))
        elif kind == 1:
            out.append((f"(= region {int(rng.integers(0, 50))})", "amount"))
        elif kind == 2:
            a = int(rng.integers(0, 45))
            out.append((f"(and (< flag {int(rng.integers(1, 100))}) (and (>= region {a}) (< region {a + 5})))", "v"))
        elif kind == 3:
            a = int(rng.integers(0, 9000))
            out.append((f"(and (>= amount {a}) (< amount {a + int(rng.integers(1, 1000))}))", None))
        elif kind == 4:
            out.append((f"(and (or (= region {int(rng.integers(0, 50))}) (= region {int(rng.integers(0, 50))})) (>= flag {int(rng.integers(0, 100))}))",
                        "amount"))
        elif kind == 5:
            out.append((f"(and (<= status {int(rng.integers(-3, 6))}) (> flag {int(rng.integers(0, 100))}))", "v"))
        else:
            out.append((f"(or (< status -1) (= region {int(rng.integers(0, 50))}))", "status"))
    return out


def _check(arrays, progs, qs, counts, sums):
    for i, (w, scol) in enumerate(qs):
        m = oracle_mask(progs[i], arrays).astype(bool)
        assert counts[i] == m.sum(), w
        if scol:
            exact = math.fsum(arrays[scol][m].astype(np.float64))
            assert abs(sums[i] - exact) <= 1e-12 * max(abs(exact), 1.0), (w, sums[i], exact)


def test_cube_answers_equal_the_oracle(env):
    ops, arrays, cols = env
    qs = _queries(np.random.default_rng(5), 140)
    progs = [ops.Program(w, cols) for w, _ in qs]
    counts, sums, prof = _run(ops, progs, [s for _, s in qs])
    assert any(k.startswith("qk_cube_") for k in prof), prof
    assert any(k.startswith("qk_cubea_") for k in prof), prof
    _check(arrays, progs, qs, counts, sums)


def test_cube_and_scan_give_the_same_integers(env):
    """A query with an f64 comparison keeps the batch's other queries on the cube but itself goes to the
    scan; the same cube-able queries alone in the per-query kernels give the same counts, and a batch of
    them plus a float-typed twin on the scan gives the same sums."""
    ops, arrays, cols = env
    qs = _queries(np.random.default_rng(6), 35)
    mixed = qs + [("(> v 20.5)", "amount"), ("(and (< v 10.0) (= region 7))", None)]
    progs = [ops.Program(w, cols) for w, _ in mixed]
    counts, sums, prof = _run(ops, progs, [s for _, s in mixed])
    assert any(k.startswith("qk_cube_") for k in prof)
    assert any(k.startswith("qk_batch_") for k in prof)
    _check(arrays, progs, mixed, counts, sums)
    for i, (w, s) in enumerate(qs[:14]):
        c, fs, _, _ = ops.fused_aggregate(progs[i], [s] if s else [])
        assert counts[i] == c, w
        if s:
            assert abs(sums[i] - fs[0]) <= 1e-12 * max(abs(fs[0]), 1.0), w


def test_few_queries_stay_on_the_scan(env):
    """Below six cube-answerable queries a table pass would cost more than the scan: the scan answers."""
    ops, arrays, cols = env
    qs = [("(< flag 7)", None), ("(= region 3)", "amount"), ("(and (>= amount 10) (< amount 900))", None)]
    progs = [ops.Program(w, cols) for w, _ in qs]
    counts, sums, prof = _run(ops, progs, [s for _, s in qs])
    assert not any(k.startswith("qk_cube") for k in prof), prof
    _check(arrays, progs, qs, counts, sums)


def test_catalog_batches_reuse_the_cube_kernels(env):
    ops, arrays, cols = env
    from computeql_gb300 import native
    lib = native.load_cuda()
    cat = ops.BatchCatalog()
    rng = np.random.default_rng(8)
    first = _queries(rng, 70)
    progs = [ops.Program(w, cols) for w, _ in first]
    c1, s1, _ = cat.aggregate(progs, [s for _, s in first])
    _check(arrays, progs, first, c1, s1)
    compiles = C.c_uint64()
    lib.cqlcuda_generated_kernel_stats(C.byref(compiles), None)
    before = compiles.value
    second = [q for i, q in enumerate(_queries(rng, 70)) if i % 7 in (0, 3, 4)]
    progs2 = [ops.Program(w, cols) for w, _ in second]
    c2, s2, _ = cat.aggregate(progs2, [s for _, s in second])
    lib.cqlcuda_generated_kernel_stats(C.byref(compiles), None)
    assert compiles.value == before
    _check(arrays, progs2, second, c2, s2)
    cat.close()


def test_values_outside_the_stated_range_fall_back_to_the_scan(env):
    ops, arrays, cols = env
    region = arrays["region"]
    narrow = ops.Column(ops.TYPE_U32, ROWS, cols["region"].buffer, zone=(0.0, 39.0), zone_map=False)   # the data reach 49
    table = dict(cols)
    table["region"] = narrow
    qs = [(f"(= region {r})", None) for r in (3, 41, 47, 12, 25, 39, 44)] + [("(< region 45)", "amount")]
    progs = [ops.Program(w, table) for w, _ in qs]
    counts, sums, prof = _run(ops, progs, [s for _, s in qs])
    assert any(k.startswith("qk_cube_") for k in prof)
    assert any(k.startswith("qk_batch_") for k in prof)   # the fallback ran the scan
    for i, (w, s) in enumerate(qs):
        m = oracle_mask(progs[i], {**arrays, "region": region}).astype(bool)
        assert counts[i] == m.sum(), w
        if s:
            assert sums[i] == float(arrays[s][m].astype(np.float64).sum()), w
