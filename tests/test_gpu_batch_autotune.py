"""The batched scan's autotuner and its 512-thread form (GB300 only).

With CQLOPS_BATCH_AUTOTUNE a plan shape's first batches each run in one candidate form (4, 8 or 16 rows a
thread at 256 threads a CTA, 8 or 16 at 512, and the tile form), timed after the candidate is compiled;
later batches of the shape run in the fastest. Every form gives the same answers, so each trial batch is
checked bit for bit against the batch in a fixed form, and every batch against the oracle.
"""
import math

import numpy as np
import pytest

from tests.batch_workload import queries, table
from tests.where_shapes import oracle_mask

pytestmark = pytest.mark.gpu
AUTOTUNE = 0xFFFFFFFF
CANDIDATES = {4 | 1 << 8, 8 | 1 << 8, 16 | 1 << 8, 8 | 2 << 8, 16 | 2 << 8, 0}


@pytest.fixture(scope="module")
def env(gpu):
    from computeql_gb300 import native, ops
    arrays = table(1_000_003, 3)
    cols = {n: ops.Column.from_numpy(a) for n, a in arrays.items()}
    return ops, native.load_ops(), arrays, cols


def test_512_thread_form_matches_the_oracle(env):
    ops, _, arrays, cols = env
    qs = queries(96, 12, 17)
    progs = [ops.Program(w, cols) for w, _ in qs]
    for form in (8 | 2 << 8, 16 | 2 << 8):
        counts, sums, _ = ops.batch_aggregate(progs, [s for _, s in qs], form)
        for i, (where, scol) in enumerate(qs):
            m = oracle_mask(progs[i], arrays).astype(bool)
            assert counts[i] == m.sum(), where
            if scol is not None:
                exact = math.fsum(arrays[scol][m])
                assert abs(sums[i] - exact) <= 1e-12 * max(abs(exact), 1e-300)


def test_autotuner_times_each_form_then_keeps_the_fastest(env):
    ops, lib, arrays, cols = env
    lib.cqlops_batch_tuner_reset()
    qs = queries(64, 8, 23)
    progs = [ops.Program(w, cols) for w, _ in qs]
    names = [s for _, s in qs]
    want_c, want_s, _ = ops.batch_aggregate(progs, names, 8)
    tried = set()
    for i in range(len(CANDIDATES)):
        c, s, _ = ops.batch_aggregate(progs, names, AUTOTUNE)
        form = lib.cqlops_batch_last_form()
        assert form >> 16 == 1, i                   # a trial
        tried.add(form & 0xFFFF)
        assert np.array_equal(c, want_c) and np.array_equal(s, want_s), form     # the same sums in every form
    assert tried == CANDIDATES
    for _ in range(3):
        c, s, _ = ops.batch_aggregate(progs, names, AUTOTUNE)
        form = lib.cqlops_batch_last_form()
        assert form >> 16 == 0 and (form & 0xFFFF) in CANDIDATES
        assert np.array_equal(c, want_c) and np.array_equal(s, want_s)
    # another plan shape (another query count bucket) is timed afresh
    more = queries(200, 8, 29)
    p2 = [ops.Program(w, cols) for w, _ in more]
    ops.batch_aggregate(p2, [s for _, s in more], AUTOTUNE)
    assert lib.cqlops_batch_last_form() >> 16 == 1
