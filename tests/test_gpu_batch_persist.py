"""The persistent shared scan (cqlops_batch_persist_*) against the launched one (GB300 only).

The persistent kernel takes each batch from a ring slot in device memory and answers into page-locked host
memory; a batch's answers must equal cqlops_batch_filter_aggregate's over the same catalog bit for bit
(the same exact integer sums, added in another order), and its counts the oracle's. Covered: batches of
varying mixes of the catalog's shapes back to back (the ring wraps several times), a kernel that reached
its idle limit between batches and is launched again, a batch with a shape new to the catalog (a new
kernel), and the stop word ending a waiting kernel at once.
"""
import time

import numpy as np
import pytest

from tests.batch_workload import F64, shapes, table
from tests.where_shapes import oracle_mask

pytestmark = pytest.mark.gpu
ROWS = 2_000_003


@pytest.fixture(scope="module")
def env(gpu):
    from computeql_gb300 import ops
    arrays = table(ROWS, 31)
    cols = {n: ops.Column.from_numpy(a) for n, a in arrays.items()}
    return ops, arrays, cols


def batch(ops, cols, gens, seed, count):
    rng = np.random.default_rng(seed)
    picks = rng.integers(0, len(gens), count)
    qs = [(gens[int(k)](rng), F64[i % 4] if i % 5 else None) for i, k in enumerate(picks)]
    return [ops.Program(w, cols) for w, _ in qs], [s for _, s in qs], qs


def test_persistent_batches_equal_launched_batches(env):
    """The launched batches run first: a device allocation or free elsewhere in the process waits for a
    running persistent kernel (until its idle limit), so the two are not interleaved here."""
    ops, arrays, cols = env
    gens = shapes(12, 77)
    cat = ops.BatchCatalog()
    progs, sums, qs = batch(ops, cols, gens, 1, 96)
    cat.aggregate(progs, sums)                     # every shape in the catalog
    batches = [batch(ops, cols, gens, seed, 40 + 13 * seed) for seed in range(2, 14)]
    want = [cat.aggregate(p, s)[:2] for p, s, _ in batches]
    # a 2 s idle limit: the oracle's checks between batches (a few hundred ms) do not let the kernel return
    with ops.PersistentScan(cat, progs, rows_per_thread=8, idle_us=2_000_000) as ps:
        for (progs, sums, qs), (want_c, want_s) in zip(batches, want):   # 12 batches: the 4-slot ring wraps three times
            got_c, got_s = ps.run(progs, sums)
            assert np.array_equal(got_c, want_c), qs[0][0]
            assert np.array_equal(got_s.view(np.uint64), want_s.view(np.uint64)), qs[0][0]
            for i in (0, len(qs) // 2, len(qs) - 1):
                assert got_c[i] == oracle_mask(progs[i], arrays).sum(), qs[i][0]
        st = ps.stats()
        assert st["batches"] == 12 and st["launches"] == 1 and st["compiles"] == 1


def test_idle_return_and_new_shape(env):
    ops, arrays, cols = env
    gens = shapes(6, 91)
    cat = ops.BatchCatalog()
    progs, sums, _ = batch(ops, cols, gens, 1, 30)
    cat.aggregate(progs, sums)
    with ops.PersistentScan(cat, progs, rows_per_thread=4, idle_us=1000) as ps:
        for seed in (2, 3):
            progs, sums, _ = batch(ops, cols, gens, seed, 30)
            got_c, got_s = ps.run(progs, sums)
            want_c, want_s, _ = cat.aggregate(progs, sums)
            assert np.array_equal(got_c, want_c) and np.array_equal(got_s.view(np.uint64), want_s.view(np.uint64))
            time.sleep(0.05)                       # 50 ms: far past the 1 ms idle limit, the kernel returns
        assert ps.stats()["launches"] >= 2
        # a shape the catalog has not met: the catalog grows and the kernel is compiled again (a batch that
        # brings a shape a summed column it had not had recompiles too)
        compiles = ps.stats()["compiles"]
        extra = [ops.Program("(and (< u0 30000) (or (>= d3 0.25) (< u2 100)))", cols)]
        progs2 = progs + extra
        sums2 = sums + ["d1"]
        got_c, got_s = ps.run(progs2, sums2)
        want_c, want_s, _ = cat.aggregate(progs2, sums2)
        assert np.array_equal(got_c, want_c) and np.array_equal(got_s.view(np.uint64), want_s.view(np.uint64))
        assert got_c[-1] == oracle_mask(extra[0], arrays).sum()
        assert ps.stats()["compiles"] == compiles + 1


def test_stop_word_ends_a_waiting_kernel(env):
    ops, _, cols = env
    gens = shapes(3, 5)
    cat = ops.BatchCatalog()
    progs, sums, _ = batch(ops, cols, gens, 1, 8)
    ps = ops.PersistentScan(cat, progs, idle_us=4_000_000)     # 4 s idle limit
    ps.run(progs, sums)
    t0 = time.monotonic()
    assert ps.close()                                           # the stop word, not the idle limit
    assert time.monotonic() - t0 < 1.0
