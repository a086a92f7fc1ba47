"""The resident chunk cache's policy (cqlops_resident_*, QE_ResidentCache of
src/query_exec/query_exec.c:1679-1970) over a host allocator (CPU only): hits and misses, generations,
which entry makes room (the most recent single-use entry first, then the least recently used), pins and
the budget."""
import ctypes as C

import numpy as np
import pytest


@pytest.fixture(scope="module")
def native():
    from computeql_gb300 import build, native as N
    build.build()
    return N


class HostDevice:
    """Buffers in host memory, so the policy runs without a GPU."""

    def __init__(self, N):
        self.N = N
        self.live = {}
        self.ops = N.CqlResidentOps(N.RESIDENT_ALLOC(self._alloc), N.RESIDENT_COPY(self._copy), N.RESIDENT_RELEASE(self._release),
                                    N.RESIDENT_MEMORY(0), N.RESIDENT_MEMORY(0), None)

    def _alloc(self, ctx, n):
        b = C.create_string_buffer(int(n))
        self.live[C.addressof(b)] = b
        return C.addressof(b)

    def _copy(self, ctx, buf, host, n):
        C.memmove(buf, host, n)
        return 1

    def _release(self, ctx, buf):
        self.live.pop(buf)


CHUNK = 100   # rows of 4 bytes: 400 bytes a chunk


def _cache(N, dev, budget):
    lib = N.load_ops()
    return lib, lib.cqlops_resident_create(budget, C.byref(dev.ops))


def _get(lib, cache, uid, gen, data, first=0, release=True):
    hit = C.c_int()
    buf = lib.cqlops_resident_acquire(cache, uid, gen, data.ctypes.data, first, CHUNK, 4, C.byref(hit))
    if buf and release:
        lib.cqlops_resident_release(cache, buf)
    return buf, bool(hit.value)


def test_miss_then_hit_and_contents(native):
    dev = HostDevice(native)
    lib, cache = _cache(native, dev, 10 * 4 * CHUNK)
    data = np.arange(CHUNK, dtype=np.uint32)
    buf, hit = _get(lib, cache, 1, 1, data)
    assert buf and not hit
    assert np.array_equal(np.frombuffer(C.string_at(buf, 4 * CHUNK), dtype=np.uint32), data)
    buf2, hit2 = _get(lib, cache, 1, 1, data)
    assert buf2 == buf and hit2
    st = lib.cqlops_resident_stats(cache)
    assert (st.hit_bytes, st.miss_bytes, st.entries, st.bytes_in_use) == (400, 400, 1, 400)
    # another generation of the column: never the old copy, which is freed when met
    buf3, hit3 = _get(lib, cache, 1, 2, data + 1)
    assert not hit3 and np.frombuffer(C.string_at(buf3, 4 * CHUNK), dtype=np.uint32)[0] == 1
    assert lib.cqlops_resident_stats(cache).entries == 1
    lib.cqlops_resident_destroy(cache)
    assert not dev.live


def test_single_use_entries_make_room_first(native):
    dev = HostDevice(native)
    lib, cache = _cache(native, dev, 10 * 4 * CHUNK)
    data = np.zeros(CHUNK, dtype=np.uint32)
    for uid in range(10):                     # A..J, each used once
        _get(lib, cache, uid, 1, data)
    for uid in (0, 1):                        # A and B used again: protected
        assert _get(lib, cache, uid, 1, data)[1]
    _get(lib, cache, 10, 1, data)             # K: the newest single-use entry (J) makes room
    assert not _get(lib, cache, 9, 1, data)[1]
    for uid in (0, 1, 2, 3):
        assert _get(lib, cache, uid, 1, data)[1], uid
    st = lib.cqlops_resident_stats(cache)
    assert st.entries == 10 and st.bytes_in_use <= 10 * 4 * CHUNK and st.evicted_bytes >= 2 * 4 * CHUNK
    lib.cqlops_resident_destroy(cache)


def test_least_recently_used_after_single_use(native):
    dev = HostDevice(native)
    lib, cache = _cache(native, dev, 3 * 4 * CHUNK)
    data = np.zeros(CHUNK, dtype=np.uint32)
    for uid in (0, 1, 2):
        _get(lib, cache, uid, 1, data)
        _get(lib, cache, uid, 1, data)        # all protected
    _get(lib, cache, 1, 1, data)              # 0 is now the least recently used
    _get(lib, cache, 3, 1, data)
    assert not _get(lib, cache, 0, 1, data)[1]
    lib.cqlops_resident_destroy(cache)


def test_pins_and_the_budget(native):
    dev = HostDevice(native)
    lib, cache = _cache(native, dev, 2 * 4 * CHUNK)
    data = np.zeros(CHUNK, dtype=np.uint32)
    a, _ = _get(lib, cache, 0, 1, data, release=False)
    b, _ = _get(lib, cache, 1, 1, data, release=False)
    c, _ = _get(lib, cache, 2, 1, data)        # both held: no room
    assert a and b and not c
    lib.cqlops_resident_release(cache, a)
    c, _ = _get(lib, cache, 2, 1, data)
    assert c
    big = np.zeros(3 * CHUNK, dtype=np.uint32)
    hit = C.c_int()
    assert not lib.cqlops_resident_acquire(cache, 9, 1, big.ctypes.data, 0, 3 * CHUNK, 4, C.byref(hit))   # larger than the budget
    assert lib.cqlops_resident_evict(cache, 1 << 30) == 4 * CHUNK        # only the unpinned one
    lib.cqlops_resident_release(cache, b)
    lib.cqlops_resident_clear(cache)
    assert lib.cqlops_resident_stats(cache).entries == 0
    lib.cqlops_resident_destroy(cache)
    assert not dev.live
