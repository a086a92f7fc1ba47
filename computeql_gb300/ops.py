"""Python face of the operator layer: device-resident columns and the operators of include/cqlops.h.

Every call goes through the C ABI (libcqlops.so -> libcqlcuda.so -> CUDA kernels). A failed call
raises with the backend's last error; nothing falls back to the CPU.
"""
from __future__ import annotations

import ctypes as C

import numpy as np

from . import native as N

TYPE_U32, TYPE_U64, TYPE_F32, TYPE_F64, TYPE_I32, TYPE_I64 = 1, 2, 3, 4, 7, 8
FUNC_COUNT, FUNC_SUM, FUNC_AVG, FUNC_MIN, FUNC_MAX = 0, 1, 2, 3, 4
CMP_EQ, CMP_LT, CMP_LE, CMP_GT, CMP_GE = 0, 1, 2, 3, 4

_NP_TYPES = {np.dtype(np.uint32): TYPE_U32, np.dtype(np.int32): TYPE_I32, np.dtype(np.float32): TYPE_F32,
             np.dtype(np.float64): TYPE_F64, np.dtype(np.uint64): TYPE_U64, np.dtype(np.int64): TYPE_I64}
_ITEM = {TYPE_U32: 4, TYPE_I32: 4, TYPE_F32: 4, TYPE_F64: 8, TYPE_U64: 8, TYPE_I64: 8}


class OpError(RuntimeError):
    pass


def _check(ok, what):
    if not ok:
        raise OpError(f"{what} failed: {N.last_error()}")


class DeviceBuffer:
    """A CqlBuffer owned by Python; released on close()/garbage collection."""

    def __init__(self, nbytes, data=None):
        lib = N.init()
        src = None
        if data is not None:
            data = np.ascontiguousarray(data)
            src = N.ptr(data)
            nbytes = data.nbytes
        self.handle = lib.cqlcuda_buffer_alloc(nbytes, 0, src)
        if not self.handle:
            raise OpError(f"cqlcuda_buffer_alloc({nbytes}) failed: {N.last_error()}")
        self.nbytes = nbytes

    def read(self, dtype, count=None):
        dtype = np.dtype(dtype)
        n = self.nbytes // dtype.itemsize if count is None else count
        out = np.empty(n, dtype=dtype)
        N.load_cuda().cqlcuda_buffer_read(self.handle, N.ptr(out), out.nbytes)
        return out

    def write(self, data):
        data = np.ascontiguousarray(data)
        N.load_cuda().cqlcuda_buffer_write(self.handle, N.ptr(data), data.nbytes)

    def close(self):
        if getattr(self, "handle", None):
            N.load_cuda().cqlcuda_buffer_release(self.handle)
            self.handle = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass


class Column:
    """A device-resident column: its buffer, CQL type, encoding and zone range."""

    def __init__(self, ctype, rows, buffer=None, width=0, base=0, zone=None):
        self.ctype = ctype
        self.rows = rows
        self.buffer = buffer
        self.width = width
        self.base = base
        self.zone = zone

    @classmethod
    def from_numpy(cls, arr, zone=True, narrow=False):
        arr = np.ascontiguousarray(arr)
        ctype = _NP_TYPES[arr.dtype]
        z = (float(arr.min()), float(arr.max())) if (zone and len(arr)) else None
        if narrow and z and ctype in (TYPE_U32, TYPE_I32):
            lo, hi = z
            span = hi - lo
            if span < 256 or span < 65536:
                w = 1 if span < 256 else 2
                base = int(lo)
                codes = (arr.astype(np.int64) - base).astype(np.uint8 if w == 1 else np.uint16)
                pad = (-codes.nbytes) % 16
                raw = np.concatenate([codes.view(np.uint8), np.zeros(pad, dtype=np.uint8)])
                return cls(ctype, len(arr), DeviceBuffer(raw.nbytes, raw), width=w, base=base & 0xFFFFFFFF, zone=z)
        return cls(ctype, len(arr), DeviceBuffer(arr.nbytes, arr), zone=z)

    @classmethod
    def sequence(cls, rows, first=0, ctype=TYPE_U32):
        return cls(ctype, rows, None, width=3, base=first & 0xFFFFFFFF, zone=(float(first), float(first + rows - 1)))

    @classmethod
    def splitmix(cls, rows, seed, per_row, index, rng):
        """u32 column draw(r*per_row+index) % rng, generated on the device."""
        buf = DeviceBuffer(rows * 4)
        _check(N.load_cuda().cqlcuda_fill_splitmix_u32(buf.handle, rows, seed, per_row, index, rng), "fill_splitmix")
        zone = (0.0, float(rng - 1)) if rng else (0.0, 4294967295.0)
        return cls(TYPE_U32, rows, buf, zone=zone)

    def c(self):
        col = N.CqlColumn()
        col.type = self.ctype
        col.width = self.width
        col.base = self.base
        col.has_range = 1 if self.zone else 0
        col.rows = self.rows
        col.buffer = self.buffer.handle if self.buffer else None
        if self.zone:
            col.zone_min, col.zone_max = self.zone
        return col


def aggregate_global(columns):
    """SUM/MIN/MAX of up to 4 columns -> (sums, mins, maxs) as lists of floats."""
    n = len(columns)
    arr = (N.CqlColumn * n)(*[c.c() for c in columns])
    s = (C.c_double * n)()
    mn = (C.c_double * n)()
    mx = (C.c_double * n)()
    _check(N.load_ops().cqlops_aggregate_global(arr, n, s, mn, mx), "cqlops_aggregate_global")
    return list(s), list(mn), list(mx)


def scan_simple(columns, leaves, want_rows=False, max_rows=None):
    """AND of (column index, op, target) leaves -> (count, sorted rows or None).
    With want_rows, at most max_rows (default: all) row numbers come back."""
    arr = (N.CqlColumn * len(columns))(*[c.c() for c in columns])
    lv = (N.CqlLeaf * len(leaves))(*[N.CqlLeaf(ci, op, float(t)) for ci, op, t in leaves])
    count = C.c_uint64()
    rows = None
    out_ptr = None
    cap = 0
    if want_rows:
        cap = columns[0].rows if max_rows is None else min(max_rows, columns[0].rows)
        rows = np.empty(max(cap, 1), dtype=np.uint32)
        out_ptr = N.ptr(rows)
    _check(N.load_ops().cqlops_scan_simple(arr, len(columns), lv, len(leaves), C.byref(count), out_ptr, cap), "cqlops_scan_simple")
    if want_rows:
        rows = rows[: min(count.value, cap)].copy()
    return count.value, rows


def group_dense(key, funcs, args):
    """Dense GROUP BY -> (min_key, counts[G], sums[G,E], mins[G,E], maxs[G,E])."""
    e = len(funcs)
    lo, hi = key.zone
    max_groups = int(hi - lo) + 1
    counts = np.zeros(max_groups, dtype=np.uint64)
    sums = np.zeros(max_groups * e, dtype=np.int64)
    mins = np.zeros(max_groups * e, dtype=np.int64)
    maxs = np.zeros(max_groups * e, dtype=np.int64)
    kc = key.c()
    # the operator layer tells argument columns apart by identity: one descriptor per distinct column
    structs = {}
    for a in args:
        if a is not None and id(a) not in structs:
            structs[id(a)] = a.c()
    col_ptrs = (C.c_void_p * e)(*[C.addressof(structs[id(a)]) if a is not None else None for a in args])
    fa = np.array(funcs, dtype=np.uint32)
    g = C.c_uint64()
    mk = C.c_int64()
    _check(N.load_ops().cqlops_group_dense(C.byref(kc), key.rows, e, N.ptr(fa), col_ptrs, max_groups, C.byref(g), C.byref(mk),
                                           N.ptr(counts), N.ptr(sums), N.ptr(mins), N.ptr(maxs)), "cqlops_group_dense")
    G = g.value
    return mk.value, counts[:G], sums[: G * e].reshape(G, e), mins[: G * e].reshape(G, e), maxs[: G * e].reshape(G, e)


def launches():
    return N.load_ops().cqlops_last_launches()
