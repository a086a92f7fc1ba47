"""The wide-table configuration's generator on the host (CPU only): its draws are the oracle's splitmix64
stream in the stated row order, and its columns have the stated ranges and distributions."""
import numpy as np

import oracle
from computeql_gb300 import workloads as w


def test_draws_follow_the_splitmix_stream():
    n = 20_000
    h, users, words = w.event_numpy(n)
    per_row = w.EVENT_DRAWS
    for i, name in enumerate(w.EVENT_U32):
        np.testing.assert_array_equal(h[name], oracle.splitmix_u32(n, w.EVENT_SEED, per_row, i, 1 << 20), err_msg=name)
    np.testing.assert_array_equal(h["user_id"], oracle.splitmix_u32(n, w.EVENT_SEED, per_row, 31, 1_000_000))
    np.testing.assert_array_equal(h["region"], oracle.splitmix_u32(n, w.EVENT_SEED, per_row, 32, 50))
    np.testing.assert_array_equal(h["status"], oracle.splitmix_u32(n, w.EVENT_SEED, per_row, 33, 5))
    np.testing.assert_array_equal(h["session"], oracle.splitmix_u32(n, w.EVENT_SEED, per_row, 38, 4_000_000))
    np.testing.assert_array_equal(users["segment"], oracle.splitmix_u32(1_000_000, w.USERS_SEED, 1, 0, 20))
    np.testing.assert_array_equal(users["user_id"], np.arange(1_000_000, dtype=np.uint32))


def test_ranges_and_distributions():
    n = 200_000
    h, _, words = w.event_numpy(n)
    for name in w.EVENT_I64:
        assert h[name].dtype == np.int64 and h[name].min() >= -(1 << 40) and h[name].max() < (1 << 40)
    for name in w.EVENT_F64:
        logs = np.log(h[name])
        assert abs(logs.mean() - 3.0) < 0.02 and abs(logs.std() - 1.0) < 0.02, name   # lognormal(3, 1)
    assert len(words) == 200 and len(set(words)) == 200
    assert all(8 <= len(x) <= 24 and x.isalpha() and x.islower() for x in words)
    for name in w.EVENT_DICT:
        counts = np.bincount(h[name], minlength=200)
        assert counts.argmax() == 0 and counts[0] > counts[1] > counts[3] > counts[10]   # Zipf, rank 1 first
        expect = (1.0 / 2.0 ** w.ZIPF_S) / 1.0
        assert abs(counts[1] / counts[0] - expect) < 0.05


def test_the_dictionary_is_fixed_by_the_seed():
    assert w.event_dictionary() == w.event_dictionary()
    assert w.event_dictionary(0) != w.event_dictionary(1)
