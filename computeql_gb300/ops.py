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
ZONEMAP_CHUNK_ROWS = 8192

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


CQLOPS_BATCH_AUTOTUNE = 0xFFFFFFFF   # rows_per_thread: the form picked per plan shape by timed trials (include/cqlops.h)


class Column:
    """A device-resident column: its buffer, CQL type, encoding and zone range."""

    def __init__(self, ctype, rows, buffer=None, width=0, base=0, zone=None, zone_map=True):
        self.ctype = ctype
        self.rows = rows
        self.buffer = buffer
        self.width = width
        self.base = base
        self.zone = zone
        self.zone_map = None
        if zone_map and buffer is not None and rows and ctype in (TYPE_U32, TYPE_I32, TYPE_F32, TYPE_F64) and width in (0, 1, 2):
            self.build_zone_map()

    def build_zone_map(self):
        """The per-chunk min/max scans prune with (8192-row chunks), computed on the GPU."""
        chunks = (self.rows + ZONEMAP_CHUNK_ROWS - 1) // ZONEMAP_CHUNK_ROWS
        zm = np.zeros(2 * (chunks + 1), dtype=np.float64)      # the chunks, then the summary pair
        self.zone_map = None
        c = self.c()
        _check(N.load_ops().cqlops_zone_map_build(C.byref(c), N.ptr(zm), chunks + 1), "cqlops_zone_map_build")
        self.zone_map = zm
        return zm

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
    def affine(cls, rows, mul, add=0, modulus=0):
        """u32 column (r * mul + add) % modulus (no reduction for modulus 0), generated on the device."""
        buf = DeviceBuffer(rows * 4)
        _check(N.load_cuda().cqlcuda_fill_affine_u32(buf.handle, rows, mul, add, modulus), "fill_affine")
        zone = (0.0, float(modulus - 1)) if modulus and modulus <= (1 << 32) else (0.0, 4294967295.0)
        return cls(TYPE_U32, rows, buf, zone=zone)

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
        if self.zone_map is not None:
            col.zone_map = self.zone_map.ctypes.data
            col.zone_map_chunks = len(self.zone_map) // 2 - 1
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


def scan_select(columns, leaves, out):
    """scan_simple with the matching rows kept on the device: up to out.nbytes // 4 of them, ascending, in the
    DeviceBuffer `out` (a selection for sort_rows, window_rank, gather_rows). -> the match count."""
    arr = (N.CqlColumn * len(columns))(*[c.c() for c in columns])
    lv = (N.CqlLeaf * len(leaves))(*[N.CqlLeaf(ci, op, float(t)) for ci, op, t in leaves])
    count = C.c_uint64()
    _check(N.load_ops().cqlops_scan_simple_select(arr, len(columns), lv, len(leaves), out.handle, C.byref(count)), "cqlops_scan_simple_select")
    return count.value


def group_dense(key, funcs, args):
    """Dense GROUP BY -> (min_key, counts[G], sums[G,E], mins[G,E], maxs[G,E])."""
    e = len(funcs)
    lo, hi = key.zone
    max_groups = int(hi - lo) + 1
    counts = np.empty(max_groups, dtype=np.uint64)
    sums = np.empty(max_groups * e, dtype=np.int64)
    mins = np.empty(max_groups * e, dtype=np.int64)
    maxs = np.empty(max_groups * e, dtype=np.int64)
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


# ---------------------------------------------------------------------------------------------
# WHERE programs, per-query kernels and fused operators

SCAN_AUTO, SCAN_INTERPRETER, SCAN_GENERATED, SCAN_SIMPLE = 0, 1, 2, 3
KERNEL_SCAN, KERNEL_FUSED_AGG, KERNEL_FUSED_GROUP = 0, 1, 2
TYPE_STRING8 = 5


class StringColumn(Column):
    """A STRING8 column: raw bytes + u64 offsets on the device, and optionally dictionary codes."""

    def __init__(self, values, dictionary=False):
        raw = [v.encode() if isinstance(v, str) else bytes(v) for v in values]
        n = len(raw)
        self.values = raw
        self.dict_struct = None
        if dictionary:
            uniq = {}
            codes = np.empty(n, dtype=np.uint32)
            for i, v in enumerate(raw):
                codes[i] = uniq.setdefault(v, len(uniq))
            items = sorted(uniq.items(), key=lambda kv: kv[1])
            offs = np.zeros(len(items) + 1, dtype=np.uint32)
            for i, (v, _) in enumerate(items):
                offs[i + 1] = offs[i] + len(v)
            blob = b"".join(v for v, _ in items) or b"\0"
            self._dict_offsets = offs
            self._dict_bytes = C.create_string_buffer(blob, len(blob))
            self.dict_struct = N.CqlDict(len(items), offs.ctypes.data, C.addressof(self._dict_bytes))
            self.codes = codes
            super().__init__(TYPE_STRING8, n, DeviceBuffer(codes.nbytes, codes) if n else DeviceBuffer(4), zone=(0.0, float(max(len(items) - 1, 0))))
            self.offsets_buf = None
        else:
            offs = np.zeros(n + 1, dtype=np.uint64)
            for i, v in enumerate(raw):
                offs[i + 1] = offs[i] + len(v)
            blob = np.frombuffer(b"".join(raw) + b"\0" * 16, dtype=np.uint8)
            super().__init__(TYPE_STRING8, n, DeviceBuffer(blob.nbytes, blob), zone=None)
            self.offsets_buf = DeviceBuffer(offs.nbytes, offs)

    @classmethod
    def from_codes(cls, codes, words):
        """A dictionary-coded column from its codes (code j is words[j]), built without a pass over the rows."""
        obj = cls.__new__(cls)
        codes = np.ascontiguousarray(codes, dtype=np.uint32)
        raw = [w.encode() if isinstance(w, str) else bytes(w) for w in words]
        offs = np.zeros(len(raw) + 1, dtype=np.uint32)
        for i, v in enumerate(raw):
            offs[i + 1] = offs[i] + len(v)
        blob = b"".join(raw) or b"\0"
        obj.values = None
        obj.codes = codes
        obj._dict_offsets = offs
        obj._dict_bytes = C.create_string_buffer(blob, len(blob))
        obj.dict_struct = N.CqlDict(len(raw), offs.ctypes.data, C.addressof(obj._dict_bytes))
        obj.offsets_buf = None
        Column.__init__(obj, TYPE_STRING8, len(codes), DeviceBuffer(codes.nbytes, codes) if len(codes) else DeviceBuffer(4),
                        zone=(0.0, float(max(len(raw) - 1, 0))))
        return obj

    def c(self):
        col = super().c()
        col.offsets = self.offsets_buf.handle if self.offsets_buf else None
        col.dict = C.addressof(self.dict_struct) if self.dict_struct else None
        return col


class Program:
    """A compiled WHERE condition over named columns (s-expression syntax, see cql_program.c)."""

    def __init__(self, where, columns):
        self.names = list(columns.keys())
        self.columns = [columns[n] for n in self.names]
        self._name_bufs = [C.create_string_buffer(n.encode()) for n in self.names]
        self._names = (C.c_char_p * len(self.names))(*[C.cast(b, C.c_char_p) for b in self._name_bufs])
        self._cols = (N.CqlColumn * len(self.columns))(*[c.c() for c in self.columns])
        self.prog = N.CqlProgram()
        ok = N.load_ops().cqlops_program_build(where.encode(), self._cols, self._names, len(self.names), C.byref(self.prog))
        if not ok:
            raise OpError("cqlops_program_build failed: " + self.prog.error.decode())

    @property
    def words(self):
        return list(self.prog.words[: self.prog.word_count])

    @property
    def consts(self):
        raw = np.array(self.prog.consts[: 2 * self.prog.const_count], dtype=np.uint32)
        return raw.view(np.float64).tolist()

    def stack_depth(self):
        return N.load_ops().cqlops_program_max_stack_depth(C.byref(self.prog))

    def source(self, kind=KERNEL_SCAN, fuse=None):
        lib = N.load_ops()
        n = C.c_uint64()
        f = C.byref(fuse) if fuse is not None else None
        if not lib.cqlops_program_source(C.byref(self.prog), kind, f, None, 0, C.byref(n)):
            why = C.create_string_buffer(256)
            lib.cqlops_program_source(C.byref(self.prog), kind, f, why, 256, None)
            raise OpError("no generated kernel: " + why.value.decode())
        buf = C.create_string_buffer(n.value + 1)
        lib.cqlops_program_source(C.byref(self.prog), kind, f, buf, n.value + 1, None)
        return buf.value.decode()

    def index(self, name):
        return self.names.index(name)


def scan_filter(program, strategy=SCAN_AUTO, want_rows=False, max_rows=None):
    """-> (count, sorted rows or None, strategy that ran)."""
    count = C.c_uint64()
    ran = C.c_uint32()
    rows_arr = None
    cap = 0
    if want_rows:
        n = program.columns[0].rows if program.columns else 0
        cap = n if max_rows is None else min(max_rows, n)
        rows_arr = np.empty(max(cap, 1), dtype=np.uint32)
    ok = N.load_ops().cqlops_scan_filter(C.byref(program.prog), program._cols, strategy, C.byref(count),
                                         N.ptr(rows_arr) if want_rows else None, cap, C.byref(ran))
    _check(ok, "cqlops_scan_filter")
    rows = rows_arr[: min(count.value, cap)].copy() if want_rows else None
    return count.value, rows, ran.value


def scan_scored(program, max_rows=None):
    """A WHERE with a fuzzy comparison (similarity / edit_distance) -> (count, rows ascending, scores)."""
    n = program.columns[0].rows if program.columns else 0
    cap = n if max_rows is None else min(max_rows, n)
    rows = np.empty(max(cap, 1), dtype=np.uint32)
    scores = np.empty(max(cap, 1), dtype=np.float64)
    count = C.c_uint64()
    _check(N.load_ops().cqlops_scan_filter_scored(C.byref(program.prog), program._cols, C.byref(count), N.ptr(rows), N.ptr(scores), cap),
           "cqlops_scan_filter_scored")
    m = min(count.value, cap)
    return count.value, rows[:m].copy(), scores[:m].copy()


def fused_aggregate(program, agg_names):
    k = len(agg_names)
    idx = (C.c_uint32 * max(k, 1))(*[program.index(n) for n in agg_names])
    cnt = C.c_double()
    s = (C.c_double * max(k, 1))()
    mn = (C.c_double * max(k, 1))()
    mx = (C.c_double * max(k, 1))()
    _check(N.load_ops().cqlops_fused_filter_aggregate(C.byref(program.prog), program._cols, idx, k, C.byref(cnt), s, mn, mx),
           "cqlops_fused_filter_aggregate")
    return cnt.value, list(s)[:k], list(mn)[:k], list(mx)[:k]


def batch_aggregate(programs, sum_names, rows_per_thread=8):
    """COUNT(*) and SUM(sum_names[q]) WHERE programs[q] for every q in one shared scan.

    All programs are built over the same columns (the first program's); sum_names[q] None = COUNT only.
    -> (counts, sums, shapes).
    """
    q = len(programs)
    base = programs[0]
    ptrs = (C.c_void_p * q)(*[C.addressof(p.prog) for p in programs])
    sc = np.array([base.index(n) if n is not None else -1 for n in sum_names], dtype=np.int32)
    counts = np.empty(max(q, 1), dtype=np.uint64)
    sums = np.empty(max(q, 1), dtype=np.float64)
    shapes = C.c_uint32()
    _check(N.load_ops().cqlops_batch_filter_aggregate(ptrs, q, base._cols, len(base.columns), N.ptr(sc), rows_per_thread, N.ptr(counts),
                                                      N.ptr(sums), C.byref(shapes)), "cqlops_batch_filter_aggregate")
    return counts[:q], sums[:q], shapes.value


def batch_source(programs, sum_names, rows_per_thread=8):
    """The generated source of the batched scan's first launch (no device work) -> (source, shapes)."""
    q = len(programs)
    base = programs[0]
    ptrs = (C.c_void_p * q)(*[C.addressof(p.prog) for p in programs])
    sc = np.array([base.index(n) if n is not None else -1 for n in sum_names], dtype=np.int32)
    n = C.c_uint64()
    shapes = C.c_uint32()
    lib = N.load_ops()
    lib.cqlops_batch_source(ptrs, q, base._cols, len(base.columns), N.ptr(sc), rows_per_thread, None, 0, C.byref(n), C.byref(shapes))
    buf = C.create_string_buffer(n.value + 1)
    _check(lib.cqlops_batch_source(ptrs, q, base._cols, len(base.columns), N.ptr(sc), rows_per_thread, buf, n.value + 1, None, None),
           "cqlops_batch_source")
    return buf.value.decode(), shapes.value


def batch_cube_source(programs, sum_names, which):
    """The cube kernels' source for these queries (which 0: the answers, 1 + p: table pass p), no device
    work -> (source, queries the cube answers); raises when no query can be answered from a cube or there
    is no such pass."""
    q = len(programs)
    base = programs[0]
    ptrs = (C.c_void_p * q)(*[C.addressof(p.prog) for p in programs])
    sc = np.array([base.index(n) if n is not None else -1 for n in sum_names], dtype=np.int32)
    n = C.c_uint64()
    nq = C.c_uint32()
    lib = N.load_ops()
    _check(lib.cqlops_batch_cube_source(ptrs, q, base._cols, len(base.columns), N.ptr(sc), which, None, 0, C.byref(n), C.byref(nq)),
           "cqlops_batch_cube_source")
    buf = C.create_string_buffer(n.value + 1)
    _check(lib.cqlops_batch_cube_source(ptrs, q, base._cols, len(base.columns), N.ptr(sc), which, buf, n.value + 1, None, None),
           "cqlops_batch_cube_source")
    return buf.value.decode(), nq.value


def fused_group(program, key_names, agg_names, max_groups=1 << 16):
    kc, ac = len(key_names), len(agg_names)
    keys = (C.c_uint32 * 3)(*[program.index(n) for n in key_names])
    aggs = (C.c_uint32 * 4)(*[program.index(n) for n in agg_names])
    total = C.c_uint64()
    kmin = (C.c_int64 * 3)()
    krange = (C.c_uint32 * 3)()
    counts = np.empty(max_groups, dtype=np.uint64)
    minrow = np.empty(max_groups, dtype=np.uint64)
    sums = np.empty(max_groups * max(ac, 1), dtype=np.int64)
    mins = np.empty(max_groups * max(ac, 1), dtype=np.int64)
    maxs = np.empty(max_groups * max(ac, 1), dtype=np.int64)
    _check(N.load_ops().cqlops_fused_filter_group(C.byref(program.prog), program._cols, keys, kc, aggs, ac, max_groups, C.byref(total), kmin,
                                                  krange, N.ptr(counts), N.ptr(minrow), N.ptr(sums), N.ptr(mins), N.ptr(maxs)),
           "cqlops_fused_filter_group")
    G = total.value
    return {"groups": G, "key_min": list(kmin)[:kc], "key_range": list(krange)[:kc], "counts": counts[:G], "min_row": minrow[:G],
            "sums": sums[: G * ac].reshape(G, ac), "mins": mins[: G * ac].reshape(G, ac), "maxs": maxs[: G * ac].reshape(G, ac)}


FUNC_ACD, FUNC_PCT = 5, 6


class HashOutputs:
    """Output arrays for group_hash kept between calls (a caller's own result area): repeated calls write into
    the same pages instead of freshly mapped ones, whose first touch costs more than the copy itself."""

    def __init__(self, max_groups, exprs):
        self.max_groups = max_groups
        self.repr_row = np.zeros(max(max_groups, 1), dtype=np.uint64)
        self.counts = np.zeros(max(max_groups, 1), dtype=np.uint64)
        self.results = np.zeros(max(max_groups, 1) * max(exprs, 1), dtype=np.float64)


def _key_values_bound(keys):
    """How many distinct key tuples the keys can form, from the whole-number keys' zone ranges (no bound
    for other keys): the most groups a GROUP BY over them can have."""
    bound = 1
    for k in keys:
        if k.ctype not in (TYPE_U32, TYPE_I32) or k.zone is None:
            return 1 << 62
        bound *= int(k.zone[1]) - int(k.zone[0]) + 1
    return bound


def group_hash(keys, funcs, args, params=None, group_hint=0, path=0, max_groups=None, out=None):
    """Hash GROUP BY -> dict(groups, repr_row[G], counts[G], results[G, E], path). With `out` (a HashOutputs)
    the results are views of its arrays, valid until its next use."""
    kc, e = len(keys), len(funcs)
    kcols = (N.CqlColumn * max(kc, 1))(*[k.c() for k in keys])
    structs = {}
    for a in args:
        if a is not None and id(a) not in structs:
            structs[id(a)] = a.c()
    arg_ptrs = (C.c_void_p * e)(*[C.addressof(structs[id(a)]) if a is not None else None for a in args])
    fa = np.array(funcs, dtype=np.uint32)
    pa = np.array(params if params is not None else [0.5] * e, dtype=np.float64)
    rows = keys[0].rows if keys else next(a.rows for a in args if a is not None)
    if out is not None:
        mg = min(out.max_groups, max_groups if max_groups is not None else out.max_groups)
        repr_row, counts, results = out.repr_row, out.counts, out.results
    else:
        mg = max_groups if max_groups is not None else min(rows, _key_values_bound(keys))
        repr_row = np.empty(max(mg, 1), dtype=np.uint64)
        counts = np.empty(max(mg, 1), dtype=np.uint64)
        results = np.empty(max(mg, 1) * e, dtype=np.float64)
    g = C.c_uint64()
    used = C.c_uint32()
    _check(N.load_ops().cqlops_group_hash(kcols, kc, e, N.ptr(fa), arg_ptrs, N.ptr(pa), group_hint, path, mg, C.byref(g), N.ptr(repr_row),
                                          N.ptr(counts), N.ptr(results), C.byref(used)), "cqlops_group_hash")
    G = g.value
    return {"groups": G, "repr_row": repr_row[:G], "counts": counts[:G], "results": results[: G * e].reshape(G, e), "path": used.value}


def group_hash_registers():
    """The HyperLogLog registers of this thread's last group_hash as a (groups * hll exprs, 1024) u32 array."""
    lib = N.load_ops()
    words = lib.cqlops_group_hash_registers(None, 0)
    out = np.empty(words, dtype=np.uint32)
    lib.cqlops_group_hash_registers(N.ptr(out), words)
    return out.reshape(-1, 1024)


def hash_join(build_key, probe_key, left=False, hint_pairs=0, want_pairs=True):
    """-> (pair count, pairs as an (n, 2) array of (probe row, build row) sorted, or None)."""
    bc, pc_ = build_key.c(), probe_key.c()
    count = C.c_uint64()
    cap = (max(probe_key.rows, build_key.rows) + probe_key.rows) * 4 if want_pairs else 0
    while True:
        out = np.empty(max(cap, 1) * 2, dtype=np.uint32) if want_pairs else None
        _check(N.load_ops().cqlops_hash_join(C.byref(bc), C.byref(pc_), 1 if left else 0, hint_pairs, C.byref(count),
                                             N.ptr(out) if want_pairs else None, cap), "cqlops_hash_join")
        n = count.value
        if not want_pairs or n <= cap:
            break
        cap = hint_pairs = n          # the host array was too small: once more with room for every pair
    return n, (out[: 2 * n].reshape(-1, 2) if want_pairs else None)


def join_aggregate(fact_key, funcs, fact_args, dim_keys, dim_rows=None, group_values=(), dim_args=None, strategy=0, dim_key_col=None,
                   dim_group_col=None):
    """Join-aggregate pushdown -> dict(groups, dim_row[G], results[G, E], strategy). dim_key_col / dim_group_col
    are the dim table's key and GROUP BY columns resident on the device (the same values as dim_keys and
    group_values[0]): a dense join then runs its dim-row pass on the device."""
    e = len(funcs)
    fk = fact_key.c()
    structs = {}
    for a in fact_args:
        if a is not None and id(a) not in structs:
            structs[id(a)] = a.c()
    fargs = (C.c_void_p * e)(*[C.addressof(structs[id(a)]) if a is not None else None for a in fact_args])
    dargs_keep = [np.ascontiguousarray(d, dtype=np.float64) if d is not None else None for d in (dim_args or [None] * e)]
    dargs = (C.c_void_p * e)(*[d.ctypes.data if d is not None else None for d in dargs_keep])
    dk = np.ascontiguousarray(dim_keys, dtype=np.uint32)
    dr = np.ascontiguousarray(dim_rows, dtype=np.uint64) if dim_rows is not None else None
    gv_keep = [np.ascontiguousarray(g, dtype=np.float64) for g in group_values]
    gv = (C.c_void_p * max(len(gv_keep), 1))(*[g.ctypes.data for g in gv_keep])
    fa = np.array(funcs, dtype=np.uint32)
    dkc = dim_key_col.c() if dim_key_col is not None else None
    dgc = dim_group_col.c() if dim_group_col is not None else None
    q = N.CqlJoinAgg(C.addressof(fk), e, fa.ctypes.data, C.addressof(fargs), C.addressof(dargs), dk.ctypes.data, len(dk),
                     dr.ctypes.data if dr is not None else None, len(dr) if dr is not None else 0, len(gv_keep),
                     C.addressof(gv) if gv_keep else None, strategy, C.addressof(dkc) if dkc is not None else None,
                     C.addressof(dgc) if dgc is not None else None)
    visits = len(dr) if dr is not None else len(dk)
    mg = max(visits, 1)
    dim_row = np.empty(mg, dtype=np.uint64)
    results = np.empty(mg * e, dtype=np.float64)
    groups = C.c_uint64()
    used = C.c_uint32()
    _check(N.load_ops().cqlops_join_aggregate(C.byref(q), mg, C.byref(groups), N.ptr(dim_row), N.ptr(results), C.byref(used)),
           "cqlops_join_aggregate")
    G = groups.value
    return {"groups": G, "dim_row": dim_row[:G], "results": results[: G * e].reshape(G, e), "strategy": used.value}


def sort_rows(keys, desc=None, selection=None, count=None, out=None):
    """ORDER BY -> row numbers in sorted order (keys compared as F64, ties by input position).

    `selection` is an optional DeviceBuffer of u32 row numbers (a filter's row set, `count` of them, all
    by default); the sort then orders those rows and returns their row numbers. `out` (optional): a u32
    array kept by the caller between calls to receive them (the result is a view of it).
    """
    kc = len(keys)
    arr = (N.CqlColumn * kc)(*[k.c() for k in keys])
    d = np.array(desc if desc is not None else [0] * kc, dtype=np.uint32)
    if selection is not None:
        n = selection.nbytes // 4 if count is None else count
        sel = selection.handle
    else:
        n, sel = keys[0].rows, None
    if out is None or len(out) < n:
        out = np.empty(max(n, 1), dtype=np.uint32)
    _check(N.load_ops().cqlops_sort_rows(arr, kc, N.ptr(d), sel, n, N.ptr(out), n), "cqlops_sort_rows")
    return out[:n]


def having(condition, columns, literals=()):
    """HAVING over grouped results: `condition` over v0..v7 (the columns, float64 arrays of one length) and
    lit[i] (the literals) -> u32 keep flags per group."""
    cols = [np.ascontiguousarray(c, dtype=np.float64) for c in columns]
    g = len(cols[0]) if cols else 0
    ptrs = (C.c_void_p * max(len(cols), 1))(*[c.ctypes.data for c in cols])
    lits = np.array(list(literals) + [0.0], dtype=np.float64)
    keep = np.empty(max(g, 1), dtype=np.uint32)
    _check(N.load_ops().cqlops_having(condition.encode(), N.ptr(lits), len(literals), ptrs, len(cols), g, N.ptr(keep)), "cqlops_having")
    return keep[:g]


WINDOW_OUTPUTS = ("rows", "row_number", "rank", "dense_rank")


def window_rank(keys, desc=None, partitions=0, selection=None, count=None, want=WINDOW_OUTPUTS, out=None):
    """ROW_NUMBER / RANK / DENSE_RANK over (PARTITION BY keys[:partitions] ORDER BY keys[partitions:])
    -> dict of u32 arrays in window order: rows, row_number, rank, dense_rank (those named in `want`; the
    others are not read back). `out` (optional): a dict of u32 arrays kept by the caller between calls to
    receive them (the results are views of them)."""
    k = len(keys)
    structs = (N.CqlColumn * k)(*[c.c() for c in keys])
    d = np.array(desc if desc is not None else [0] * k, dtype=np.uint32)
    if selection is not None:
        n = selection.nbytes // 4 if count is None else count
    else:
        n = keys[0].rows
    arrays = {}
    for name in want:
        a = out.get(name) if out is not None else None
        if a is None or len(a) < max(n, 1):
            a = np.empty(max(n, 1), dtype=np.uint32)
            if out is not None:
                out[name] = a
        arrays[name] = a
    ptr = lambda name: N.ptr(arrays[name]) if name in arrays else None
    _check(N.load_ops().cqlops_window_rank(structs, k, N.ptr(d), partitions, selection.handle if selection is not None else None, n,
                                           ptr("rows"), ptr("row_number"), ptr("rank"), ptr("dense_rank"), max(n, 1)),
           "cqlops_window_rank")
    return {name: a[:n] for name, a in arrays.items()}


_GATHER_DTYPES = {TYPE_U32: np.uint32, 12: np.uint32, TYPE_I32: np.int32, 9: np.int32, TYPE_F32: np.float32, TYPE_U64: np.uint64,
                  TYPE_I64: np.int64, 10: np.int64, 11: np.int64, TYPE_F64: np.float64, 6: np.uint8, TYPE_STRING8: np.uint32}


def _gather_selection(rows, selection, count, default):
    if rows is not None:
        r = np.ascontiguousarray(rows, dtype=np.uint32)
        return r, None, len(r)
    if selection is not None:
        return None, selection, (selection.nbytes // 4 if count is None else count)
    return None, None, (default if count is None else count)


def gather_rows(columns, rows=None, selection=None, count=None):
    """Row materialization: the selected rows' values of each column, in selection order -> a list of
    arrays (narrow and sequence columns decoded, dictionary strings as their codes). The selection is
    `rows` (host row numbers), else the device buffer `selection`, else rows 0..count-1."""
    k = len(columns)
    r, sel, n = _gather_selection(rows, selection, count, min((c.rows for c in columns), default=0))
    # one host block, each column at its offset in the device's gather area, so that it comes back in one read
    dtypes = [np.dtype(_GATHER_DTYPES[c.ctype]) for c in columns]
    offsets, total = [], 0
    for dt in dtypes:
        offsets.append(total)
        total += (max(n, 1) * dt.itemsize + 15) & ~15
    block = np.empty(max(total, 16), dtype=np.uint8)
    outs = [block[o:o + max(n, 1) * dt.itemsize].view(dt) for o, dt in zip(offsets, dtypes)]
    structs = (N.CqlColumn * k)(*[c.c() for c in columns])
    ptrs = (C.c_void_p * k)(*[o.ctypes.data for o in outs])
    _check(N.load_ops().cqlops_gather_rows(structs, k, N.ptr(r) if r is not None else None, sel.handle if sel is not None else None, n, ptrs),
           "cqlops_gather_rows")
    return [o[:n] for o in outs]


def gather_strings(column, rows=None, selection=None, count=None):
    """The selected rows of a raw string column -> a list of bytes objects, in selection order."""
    r, sel, n = _gather_selection(rows, selection, count, column.rows)
    offs = np.zeros(n + 1, dtype=np.uint64)
    lib = N.load_ops()
    c = column.c()
    need = C.c_uint64()
    cap = 0
    buf = C.create_string_buffer(1)
    for _ in range(2):
        ok = lib.cqlops_gather_strings(C.byref(c), N.ptr(r) if r is not None else None, sel.handle if sel is not None else None, n,
                                       N.ptr(offs), buf, cap, C.byref(need))
        if ok:
            data = buf.raw
            return [data[int(offs[i]):int(offs[i + 1])] for i in range(n)]
        if need.value <= cap:
            break
        cap = need.value
        buf = C.create_string_buffer(max(cap, 1))
    _check(0, "cqlops_gather_strings")


def fixed_scale(column, selection=None, count=None):
    """-> (scale or -1, largest magnitude): the decimal places every value needs (at most 6)."""
    n = column.rows if selection is None else (selection.nbytes // 4 if count is None else count)
    c = column.c()
    scale = C.c_int32()
    largest = C.c_double()
    _check(N.load_ops().cqlops_fixed_scale(C.byref(c), selection.handle if selection is not None else None, n, C.byref(scale),
                                           C.byref(largest)), "cqlops_fixed_scale")
    return scale.value, largest.value


def group_dense_fixed(key, funcs, args, selection=None, count=None, max_groups=65536):
    """GROUP BY key with COUNT/SUM/AVG/MIN/MAX over decimal f64/f32 columns, exact as scaled integers.

    -> dict(keys, first_rows, counts, results[G, E], scales) for the present groups in key order.
    """
    e = len(funcs)
    kc = key.c()
    structs = [a.c() if a is not None else None for a in args]
    arr = (C.c_void_p * e)(*[C.addressof(s) if s is not None else None for s in structs])
    fa = np.array(funcs, dtype=np.uint32)
    n = key.rows if selection is None else (selection.nbytes // 4 if count is None else count)
    keys = np.empty(max_groups, dtype=np.int64)
    first = np.empty(max_groups, dtype=np.uint64)
    counts = np.empty(max_groups, dtype=np.uint64)
    results = np.empty(max_groups * e, dtype=np.float64)
    scales = np.zeros(e, dtype=np.int32)
    groups = C.c_uint64()
    _check(N.load_ops().cqlops_group_dense_fixed(C.byref(kc), e, N.ptr(fa), arr, selection.handle if selection is not None else None,
                                                 n, max_groups, C.byref(groups), N.ptr(keys), N.ptr(first), N.ptr(counts),
                                                 N.ptr(results), N.ptr(scales)), "cqlops_group_dense_fixed")
    G = groups.value
    return {"keys": keys[:G], "first_rows": first[:G], "counts": counts[:G], "results": results[: G * e].reshape(G, e),
            "scales": list(scales)}


def compile_check(source):
    """NVRTC compile of a generated source for sm_103a, no device needed -> (ok, log)."""
    lib = N.load_cuda()
    b = source.encode()
    ok = lib.cqlcuda_compile_check(b, len(b))
    log = lib.cqlcuda_last_compile_log()
    return bool(ok), (log.decode() if log else "")


# ---------------------------------------------------------------------------------------------
# the served form (include/cqlserve.h)

SERVE_FILTER_AGG, SERVE_AGG_GLOBAL, SERVE_GROUP_DENSE, SERVE_CALL = 1, 2, 3, 4
_SERVE_CALL = C.CFUNCTYPE(C.c_int, C.c_void_p)


class BatchCatalog:
    """A shape catalog for repeated shared scans over one table (cqlops_batch_catalog_*)."""

    def __init__(self):
        self.h = N.load_ops().cqlops_batch_catalog_create()
        if not self.h:
            raise OpError("cqlops_batch_catalog_create failed")

    @property
    def shapes(self):
        return N.load_ops().cqlops_batch_catalog_shapes(self.h)

    def aggregate(self, programs, sum_names, rows_per_thread=8):
        """batch_aggregate through the catalog -> (counts, sums, shapes)."""
        q = len(programs)
        base = programs[0]
        ptrs = (C.c_void_p * q)(*[C.addressof(p.prog) for p in programs])
        sc = np.array([base.index(n) if n is not None else -1 for n in sum_names], dtype=np.int32)
        counts = np.empty(max(q, 1), dtype=np.uint64)
        sums = np.empty(max(q, 1), dtype=np.float64)
        shapes = C.c_uint32()
        _check(N.load_ops().cqlops_batch_filter_aggregate_cat(self.h, ptrs, q, base._cols, len(base.columns), N.ptr(sc), rows_per_thread,
                                                              N.ptr(counts), N.ptr(sums), C.byref(shapes)), "cqlops_batch_filter_aggregate_cat")
        return counts[:q], sums[:q], shapes.value

    def close(self):
        if self.h:
            N.load_ops().cqlops_batch_catalog_destroy(self.h)
            self.h = None


class PersistentScan:
    """The persistent shared scan over one table (cqlops_batch_persist_*): one long-lived kernel that takes
    batches from a ring of parameter slots in device memory. The catalog must outlive it."""

    def __init__(self, catalog, programs, rows_per_thread=8, idle_us=2000):
        base = programs[0]
        self.catalog = catalog
        self._cols = base._cols
        self._names = base
        self.h = N.load_ops().cqlops_batch_persist_create(catalog.h, base._cols, len(base.columns), rows_per_thread, idle_us)
        if not self.h:
            raise OpError("cqlops_batch_persist_create: " + N.load_ops().cqlops_last_error().decode())

    def run(self, programs, sum_names):
        """-> (counts, sums) of the batch, as batch_aggregate's"""
        q = len(programs)
        base = programs[0]
        ptrs = (C.c_void_p * q)(*[C.addressof(p.prog) for p in programs])
        sc = np.array([base.index(n) if n is not None else -1 for n in sum_names], dtype=np.int32)
        counts = np.empty(max(q, 1), dtype=np.uint64)
        sums = np.empty(max(q, 1), dtype=np.float64)
        _check(N.load_ops().cqlops_batch_persist_run(self.h, ptrs, q, N.ptr(sc), N.ptr(counts), N.ptr(sums)), "cqlops_batch_persist_run")
        return counts[:q], sums[:q]

    def stats(self):
        b, l, c = C.c_uint64(), C.c_uint64(), C.c_uint64()
        N.load_ops().cqlops_batch_persist_stats(self.h, C.byref(b), C.byref(l), C.byref(c))
        return {"batches": b.value, "launches": l.value, "compiles": c.value, "ctas": N.load_ops().cqlops_batch_persist_ctas(self.h)}

    def close(self):
        if self.h:
            ok = N.load_ops().cqlops_batch_persist_destroy(self.h)
            self.h = None
            return bool(ok)
        return True

    def __enter__(self):
        return self

    def __exit__(self, *exc):
        self.close()

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass


class ServeTable:
    """A table registered with a Server: its named columns, in the order programs over it must use."""

    def __init__(self, index, columns):
        self.index = index
        self.names = list(columns.keys())
        self.columns = columns

    def col(self, name):
        return self.names.index(name)

    def program(self, where):
        return Program(where, self.columns)


class ServeRequest:
    """A submitted request; wait() blocks until it is done, then the result fields are valid."""

    def __init__(self, server, req, keep):
        self.server = server
        self.req = req
        self._keep = keep

    def wait(self, timeout_ms=0):
        return bool(N.load_ops().cqlserve_wait(self.server.h, C.byref(self.req), timeout_ms))

    @property
    def status(self):
        return self.req.status

    @property
    def ok(self):
        return self.req.status == 1

    @property
    def error(self):
        return self.req.error.decode()

    @property
    def count(self):
        return self.req.count

    @property
    def sum(self):
        return self.req.sum[0]

    @property
    def fused(self):
        return self.req.fused

    @property
    def latency_ns(self):
        return self.req.done_ns - self.req.submit_ns

    def group_result(self):
        g = self.req.count
        e = self.req.expr_count
        counts, sums, mins, maxs = self._keep[1:5]
        return (self.req.min_key, counts[:g], sums[: g * e].reshape(g, e), mins[: g * e].reshape(g, e), maxs[: g * e].reshape(g, e))


class Server:
    """Concurrent serving over resident tables: worker threads on their own lanes, admission by planned
    device footprint, and (fuse=True) continuous batching of filter/aggregate requests into shared scans."""

    def __init__(self, workers=2, fuse=True, max_fuse=1024, rows_per_thread=8, memory_budget=0):
        cfg = N.CqlServeConfig(workers, int(bool(fuse)), max_fuse, rows_per_thread, memory_budget)
        self.h = N.load_ops().cqlserve_create(C.byref(cfg))
        if not self.h:
            raise OpError("cqlserve_create failed: " + N.last_error())
        self._tables = []

    def add_table(self, columns):
        arr = (N.CqlColumn * len(columns))(*[c.c() for c in columns.values()])
        idx = N.load_ops().cqlserve_add_table(self.h, arr, len(columns))
        if idx < 0:
            raise OpError("cqlserve_add_table failed")
        t = ServeTable(idx, columns)
        t._arr = arr
        self._tables.append(t)
        return t

    def prepare(self, table, programs, sum_names):
        q = len(programs)
        ptrs = (C.c_void_p * q)(*[C.addressof(p.prog) for p in programs])
        sc = np.array([table.col(n) if n is not None else -1 for n in sum_names], dtype=np.int32)
        _check(N.load_ops().cqlserve_prepare(self.h, table.index, ptrs, q, N.ptr(sc)), "cqlserve_prepare")

    def _submit(self, req, keep, submit=True):
        r = ServeRequest(self, req, keep)
        if submit:
            N.load_ops().cqlserve_submit(self.h, C.byref(req))
        return r

    def submit(self, request):
        """Queues a request built with submit=False."""
        N.load_ops().cqlserve_submit(self.h, C.byref(request.req))
        return request

    def filter_agg(self, table, program, sum_name=None, submit=True):
        """SELECT COUNT(*)[, SUM(sum_name)] WHERE program."""
        if program.names != table.names:
            raise OpError("the program is not built over the table's columns")
        req = N.CqlServeRequest()
        req.kind = SERVE_FILTER_AGG
        req.table = table.index
        req.program = C.addressof(program.prog)
        req.sum_column = table.col(sum_name) if sum_name is not None else -1
        return self._submit(req, (program,), submit)

    def agg_global(self, table, names, submit=True):
        """SUM/MIN/MAX of up to 4 columns."""
        req = N.CqlServeRequest()
        req.kind = SERVE_AGG_GLOBAL
        req.table = table.index
        req.column_count = len(names)
        for i, n in enumerate(names):
            req.columns[i] = table.col(n)
        return self._submit(req, (), submit)

    def group_dense(self, table, key, funcs, args, submit=True):
        """GROUP BY key (small range) with funcs over args (None for COUNT)."""
        e = len(funcs)
        lo, hi = table.columns[key].zone
        g = int(hi - lo) + 1
        counts = np.empty(g, dtype=np.uint64)
        sums = np.empty(g * e, dtype=np.int64)
        mins = np.empty(g * e, dtype=np.int64)
        maxs = np.empty(g * e, dtype=np.int64)
        req = N.CqlServeRequest()
        req.kind = SERVE_GROUP_DENSE
        req.table = table.index
        req.column_count = 1
        req.columns[0] = table.col(key)
        req.expr_count = e
        for i, (f, a) in enumerate(zip(funcs, args)):
            req.funcs[i] = f
            req.args[i] = table.col(a) if a is not None else -1
        req.max_groups = g
        req.out_counts, req.out_sums, req.out_mins, req.out_maxs = (a.ctypes.data for a in (counts, sums, mins, maxs))
        return self._submit(req, ((), counts, sums, mins, maxs), submit)

    def call(self, fn, footprint=0):
        """Runs fn() (-> bool) on a worker, admitted with `footprint` planned device bytes."""
        cb = _SERVE_CALL(lambda _ctx: 1 if fn() else 0)
        req = N.CqlServeRequest()
        req.kind = SERVE_CALL
        req.call = C.cast(cb, C.c_void_p)
        req.footprint = footprint
        return self._submit(req, (cb,))

    def join(self, fact_key, funcs, fact_args, dim_keys, dim_rows=None, group_values=(), dim_key_col=None, dim_group_col=None,
             footprint=1 << 20, submit=True):
        """A join-aggregate (cqlops_join_aggregate) as a native call request: no Python runs on the worker.
        The result is in .req.ctx's CqlServeJoin (see join_result)."""
        e = len(funcs)
        keep = {"fk": fact_key.c()}
        structs = {}
        for a in fact_args:
            if a is not None and id(a) not in structs:
                structs[id(a)] = a.c()
        keep["structs"] = structs
        keep["fargs"] = (C.c_void_p * e)(*[C.addressof(structs[id(a)]) if a is not None else None for a in fact_args])
        keep["dk"] = np.ascontiguousarray(dim_keys, dtype=np.uint32)
        keep["dr"] = np.ascontiguousarray(dim_rows, dtype=np.uint64) if dim_rows is not None else None
        keep["gv"] = [np.ascontiguousarray(g, dtype=np.float64) for g in group_values]
        keep["gvp"] = (C.c_void_p * max(len(keep["gv"]), 1))(*[g.ctypes.data for g in keep["gv"]])
        keep["fa"] = np.array(funcs, dtype=np.uint32)
        keep["dkc"] = dim_key_col.c() if dim_key_col is not None else None
        keep["dgc"] = dim_group_col.c() if dim_group_col is not None else None
        visits = len(keep["dr"]) if keep["dr"] is not None else len(keep["dk"])
        keep["rows"] = np.empty(max(visits, 1), dtype=np.uint64)
        keep["res"] = np.empty(max(visits, 1) * e, dtype=np.float64)
        q = N.CqlJoinAgg(C.addressof(keep["fk"]), e, keep["fa"].ctypes.data, C.addressof(keep["fargs"]), None, keep["dk"].ctypes.data,
                         len(keep["dk"]), keep["dr"].ctypes.data if keep["dr"] is not None else None,
                         len(keep["dr"]) if keep["dr"] is not None else 0, len(keep["gv"]),
                         C.addressof(keep["gvp"]) if keep["gv"] else None, 0,
                         C.addressof(keep["dkc"]) if keep["dkc"] is not None else None,
                         C.addressof(keep["dgc"]) if keep["dgc"] is not None else None)
        ctx = N.CqlServeJoin(q, max(visits, 1), keep["rows"].ctypes.data, keep["res"].ctypes.data, 0, 0)
        keep["ctx"] = ctx
        return self._native_call("cqlserve_join_call", ctx, footprint, keep, submit)

    def sort(self, columns, leaves, sort_column, desc, limit, max_rows, footprint=0, submit=True):
        """SELECT ... WHERE <leaves> ORDER BY columns[sort_column] [DESC] LIMIT limit as a native call request."""
        keep = {"cols": (N.CqlColumn * len(columns))(*[c.c() for c in columns]),
                "leaves": (N.CqlLeaf * len(leaves))(*[N.CqlLeaf(ci, op, float(t)) for ci, op, t in leaves]),
                "out": np.zeros(max(limit, 1), dtype=np.uint32)}
        ctx = N.CqlServeSort(C.addressof(keep["cols"]), len(columns), C.addressof(keep["leaves"]), len(leaves), sort_column,
                             1 if desc else 0, max_rows, limit, keep["out"].ctypes.data, 0)
        keep["ctx"] = ctx
        return self._native_call("cqlserve_sort_call", ctx, footprint or max_rows * 32, keep, submit)

    def _native_call(self, fn_name, ctx, footprint, keep, submit):
        req = N.CqlServeRequest()
        req.kind = SERVE_CALL
        req.call = C.cast(getattr(N.load_ops(), fn_name), C.c_void_p)
        req.ctx = C.addressof(ctx)
        req.footprint = footprint
        return self._submit(req, keep, submit)

    def drain(self):
        N.load_ops().cqlserve_drain(self.h)

    def stats(self):
        s = N.load_ops().cqlserve_stats(self.h)
        return {n: getattr(s, n) for n, _ in N.CqlServeStats._fields_}

    def close(self):
        if self.h:
            N.load_ops().cqlserve_destroy(self.h)
            self.h = None

    def __enter__(self):
        return self

    def __exit__(self, *exc):
        self.close()

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass
