"""The slot compaction that allocates nothing, against the aggregate_compact entry point.

Callers that cannot allocate device memory mid-query (a serving loop that has committed all of HBM to
resident tables and per-query budgets) use cqlcuda_compact_slots_noalloc. It runs the three
aggregate_compact passes over the caller's own buffers, with the block totals in a static device
array. Both paths go through the C ABI here, on two calls in a row with different slot tables, and
must agree exactly (the outputs are whole numbers). This file is collected last on purpose.
"""
import ctypes as C

import numpy as np
import pytest

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def lib(gpu):
    return gpu.load_cuda()


def device_buffer(lib, nbytes, data=None):
    src = C.c_void_p(data.ctypes.data) if data is not None else None
    h = lib.cqlcuda_buffer_alloc(nbytes, 0, src)
    assert h, lib.cqlcuda_last_error()
    return h


def reference_compact(lib, counts, owner):
    """aggregate_compact by name, three dispatches in one batch, through the backend ABI"""
    n = len(counts)
    blocks = (n + 255) // 256
    k = lib.cqlcuda_kernel_alloc(b"aggregate_compact", 17)
    bufs = [device_buffer(lib, n * 4, counts), device_buffer(lib, n * 4, owner), device_buffer(lib, (n + 1) * 4),
            device_buffer(lib, blocks * 4), device_buffer(lib, n * 4), device_buffer(lib, n * 4), device_buffer(lib, 4)]
    for i, b in enumerate(bufs):
        lib.cqlcuda_kernel_set_arg_buffer(k, i, b)
    lib.cqlcuda_kernel_set_arg_u64(k, 0, n)
    offsets = np.zeros(n + 1, dtype=np.uint32)
    g_owner = np.zeros(n, dtype=np.uint32)
    g_count = np.zeros(n, dtype=np.uint32)
    total = np.zeros(1, dtype=np.uint32)
    batch = lib.cqlcuda_batch_begin(0, 0)
    for mode, gws in ((0, blocks * 256), (1, 256), (2, blocks * 256)):
        lib.cqlcuda_kernel_set_arg_u64(k, 1, mode)
        lib.cqlcuda_batch_kernel_execute(batch, k, gws, 256)
    for b, arr in ((bufs[2], offsets), (bufs[4], g_owner), (bufs[5], g_count), (bufs[6], total)):
        lib.cqlcuda_batch_buffer_read(batch, b, C.c_void_p(arr.ctypes.data), arr.nbytes)
    assert lib.cqlcuda_batch_end(batch) == 1
    for b in bufs:
        lib.cqlcuda_buffer_release(b)
    return offsets, g_owner, g_count, int(total[0])


class NoallocCase:
    """Inputs and outputs of one slot table in device buffers the caller owns."""

    def __init__(self, lib, counts, owner):
        self.lib, self.n = lib, len(counts)
        n = self.n
        self.ins = [device_buffer(lib, n * 4, counts), device_buffer(lib, n * 4, owner)]
        self.outs = [device_buffer(lib, (n + 1) * 4), device_buffer(lib, n * 4), device_buffer(lib, n * 4)]

    def run(self):
        lib, n, ptr = self.lib, self.n, self.lib.cqlcuda_buffer_device_pointer
        total = C.c_uint32(0)
        rc = lib.cqlcuda_compact_slots_noalloc(ptr(self.ins[0]), ptr(self.ins[1]), n, ptr(self.outs[0]), ptr(self.outs[1]),
                                               ptr(self.outs[2]), C.byref(total), None)
        assert rc == 1, (rc, lib.cqlcuda_last_error())
        offsets = np.zeros(n + 1, dtype=np.uint32)
        g_owner = np.zeros(n, dtype=np.uint32)
        g_count = np.zeros(n, dtype=np.uint32)
        for b, arr in zip(self.outs, (offsets, g_owner, g_count)):
            lib.cqlcuda_buffer_read(b, C.c_void_p(arr.ctypes.data), arr.nbytes)
        return offsets, g_owner, g_count, total.value

    def release(self):
        for b in self.ins + self.outs:
            self.lib.cqlcuda_buffer_release(b)


def noalloc_compact(lib, counts, owner):
    case = NoallocCase(lib, counts, owner)
    try:
        return case.run()
    finally:
        case.release()


def slot_table(n, occupancy, seed):
    rng = np.random.default_rng(seed)
    counts = np.where(rng.random(n) < occupancy, rng.integers(1, 50, n), 0).astype(np.uint32)
    owner = np.where(counts > 0, rng.integers(0, 1 << 30, n), 0xFFFFFFFF).astype(np.uint32)
    return counts, owner


def test_two_calls_in_a_row_match_the_existing_entry_point(lib):
    for n, occupancy, seed in ((1_048_576 + 123, 0.3, 1), (70_001, 0.9, 2)):
        counts, owner = slot_table(n, occupancy, seed)
        ref = reference_compact(lib, counts, owner)
        got = noalloc_compact(lib, counts, owner)
        total = ref[3]
        assert got[3] == total == int((counts > 0).sum())
        occupied = counts > 0
        assert np.array_equal(got[0][:n][occupied], ref[0][:n][occupied])
        assert got[0][n] == ref[0][n] == total
        assert np.array_equal(got[1][:total], ref[1][:total])
        assert np.array_equal(got[2][:total], ref[2][:total])
        assert np.array_equal(got[2][:total], counts[occupied])


def test_device_memory_does_not_move_across_calls(lib):
    """With its buffers in place, calls after the first leave the device's free memory where it was:
    the entry point allocates nothing and loads no module (the library's init resolved its scratch)."""
    counts, owner = slot_table(1 << 20, 0.5, 3)
    case = NoallocCase(lib, counts, owner)
    try:
        first = case.run()
        free0 = lib.cqlcuda_device_free_memory()
        for _ in range(3):
            got = case.run()
            assert got[3] == first[3]
            assert np.array_equal(got[1][: got[3]], first[1][: first[3]])
        assert lib.cqlcuda_device_free_memory() == free0
    finally:
        case.release()


def test_rejects_sizes_past_its_limit_and_null_pointers(lib):
    dummy = C.c_void_p(1)
    total = C.c_uint32(0)
    assert lib.cqlcuda_compact_slots_noalloc(dummy, dummy, (1 << 24) + 1, dummy, dummy, dummy, C.byref(total), None) == -1
    assert b"it takes 1 to 16777216" in lib.cqlcuda_last_error()
    assert lib.cqlcuda_compact_slots_noalloc(dummy, dummy, 0, dummy, dummy, dummy, C.byref(total), None) == -1
    assert lib.cqlcuda_compact_slots_noalloc(None, dummy, 16, dummy, dummy, dummy, C.byref(total), None) == -2
    assert b"NULL pointer" in lib.cqlcuda_last_error()
