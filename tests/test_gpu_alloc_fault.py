"""Allocation failure at every allocation of a query: each run is right or fails cleanly (GB300 only).

The reference's contract, src/tests/bench_alloc_fault.c:380-430: a query is run cold once to count its
allocation attempts; then for every k it is run cold again with the k-th allocation failing
(g_gpu_fault_alloc_at, src/gpu/gpu.h:68 - here cqlcuda_set_fault_alloc_at). Each injected run must either
return the reference answer or report an error, never a wrong answer; and the next run without injection
must be right again. "Cold" drops the backend's pooled buffers first (cqlcuda_pool_evict, as the
reference's af_drop_caches, :236-241), so every pooled allocation happens again. The failure is made on
the host, in the allocator: no kernel runs with a missing buffer.
"""
import numpy as np
import pytest

import oracle

pytestmark = pytest.mark.gpu
COUNT, SUM, AVG, MIN, MAX = 0, 1, 2, 3, 4
N = 1_000_003


@pytest.fixture(scope="module")
def env(gpu):
    from computeql_gb300 import ops, workloads
    t = workloads.fact_table(N)
    h = workloads.fact_numpy(N, gen=oracle.splitmix_u32)
    rng = np.random.default_rng(11)
    hkey = rng.integers(0, 200_000, N).astype(np.uint32)
    key = ops.Column.from_numpy(hkey)
    val = ops.Column.from_numpy(rng.integers(0, 1_000_000, N).astype(np.uint32))
    dk = np.arange(1_000_000, dtype=np.uint32)
    seg = oracle.splitmix_u32(1_000_000, workloads.DIM1M_SEED, 1, 0, 20).astype(np.float64)
    prog = ops.Program("(or (< flag 3) (and (> amount 9000) (= region 7)))", {"flag": t.flag, "amount": t.amount, "region": t.region})
    measure = ops.Column.from_numpy(rng.lognormal(3.0, 1.0, N))
    return ops, gpu.load_cuda(), t, h, key, val, dk, seg, prog, hkey, measure


def by_key(res, hkey):
    """a hash GROUP BY's groups keyed by their key value: the order of its groups and the row that
    represents each are whichever slot claim won, in the reference too"""
    keys = hkey[res["repr_row"].astype(np.int64)]
    return sorted(zip(keys.tolist(), res["counts"].tolist(), res["results"].tolist()))


def queries(env):
    ops, _, t, _, key, val, dk, seg, prog, hkey, measure = env

    def select_then_sort():
        sel = ops.DeviceBuffer(N * 4)
        n = ops.scan_select([t.flag], [(0, ops.CMP_LT, 2)], sel)
        return n, ops.sort_rows([t.amount], selection=sel, count=n)

    return {
        "aggregate_global": lambda: ops.aggregate_global([t.amount]),
        "scan_simple_rows": lambda: ops.scan_simple([t.flag], [(0, ops.CMP_LT, 2)], want_rows=True),
        "scan_filter_generated": lambda: ops.scan_filter(prog, strategy=ops.SCAN_GENERATED, want_rows=True),
        "group_dense": lambda: ops.group_dense(t.region, [SUM, COUNT, MIN, MAX], [t.amount, None, t.amount, t.amount]),
        "group_hash": lambda: by_key(ops.group_hash([key], [COUNT, SUM], [None, val]), hkey),
        # a failed allocation may move the join to another strategy (dense core to probe); the answer must hold
        "join_aggregate": lambda: {k: v for k, v in ops.join_aggregate(t.amount, [SUM, COUNT], [t.amount, None], dk,
                                                                      group_values=[seg]).items() if k != "strategy"},
        "sort_rows": lambda: ops.sort_rows([key]),
        # the one-pass small-key GROUP BY over an f64 measure, and a filter's rows kept on the device for a sort
        "group_small": lambda: ops.group_hash([t.region], [SUM, AVG, MIN, MAX], [measure] * 4),
        "scan_select_sort": select_then_sort,
    }


def canon(x):
    """A result as nested plain values, comparable with ==."""
    if isinstance(x, dict):
        return {k: canon(v) for k, v in x.items()}
    if isinstance(x, (list, tuple)):
        return [canon(v) for v in x]
    if isinstance(x, np.ndarray):
        return x.tolist()
    return x


def drop_caches(lib):
    """af_drop_caches (bench_alloc_fault.c:236-241): a new pool epoch, then every pooled buffer evicted"""
    lib.cqlcuda_pool_begin_epoch()
    lib.cqlcuda_pool_evict(2 ** 64 - 1)


def run(fn):
    from computeql_gb300 import native, ops
    try:
        return "ok", canon(fn())
    except (ops.OpError, native.CudaError) as e:
        return "error", str(e)


@pytest.mark.parametrize("name", ["aggregate_global", "scan_simple_rows", "scan_filter_generated", "group_dense", "group_hash",
                                  "join_aggregate", "sort_rows", "group_small", "scan_select_sort"])
def test_every_allocation_fails_cleanly(env, name):
    ops, lib = env[0], env[1]
    fn = queries(env)[name]
    status, reference = run(fn)
    assert status == "ok", reference
    drop_caches(lib)
    before = lib.cqlcuda_memory_stats().alloc_calls
    status, cold = run(fn)
    allocations = lib.cqlcuda_memory_stats().alloc_calls - before
    assert status == "ok" and cold == reference
    assert allocations > 0, "a cold run allocates"
    tally = {"correct": 0, "error": 0, "unreached": 0}
    for k in range(1, allocations + 1):
        drop_caches(lib)
        target = lib.cqlcuda_memory_stats().alloc_calls + k
        lib.cqlcuda_set_fault_alloc_at(target)
        try:
            status, got = run(fn)
            fired = lib.cqlcuda_memory_stats().alloc_calls >= target
        finally:
            lib.cqlcuda_set_fault_alloc_at(0)
        if not fired:
            tally["unreached"] += 1
        elif status == "error":
            tally["error"] += 1
        else:
            assert got == reference, f"{name}: allocation {k} of {allocations} failed and the answer is wrong"
            tally["correct"] += 1
        status, after = run(fn)
        assert status == "ok" and after == reference, f"{name}: the run after a failed allocation {k} is not right"
    assert tally["error"] + tally["correct"] + tally["unreached"] == allocations
    # the injected failures were met; each gave an error or, where an operator has another path (the join's
    # dense core falls back to the probe), the right answer
    assert tally["error"] + tally["correct"] > 0, tally
