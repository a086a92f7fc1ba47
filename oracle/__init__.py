"""CPU oracle: a C restatement of the reference's algorithms, loaded with ctypes.

TEST INFRASTRUCTURE ONLY. Only tests/, __graft_entry__.smoke() and bench.py's cpu_baseline leg
(and its --impl reference arm) may import this package; the product never does.
"""
from __future__ import annotations

import ctypes as C
import os
import subprocess

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
LIB = os.path.join(HERE, "_build", "liboracle.so")
SOURCES = [os.path.join(HERE, "oracle.c"), os.path.join(HERE, "oracle_sketch.c"), os.path.join(HERE, "oracle_sort.c"),
           os.path.join(HERE, "oracle_join.c"), os.path.join(HERE, "oracle_fixed.c")]

U32, U64, F32, F64, I32, I64 = 1, 2, 3, 4, 7, 8

_lib = None


def build():
    os.makedirs(os.path.dirname(LIB), exist_ok=True)
    deps = SOURCES + [os.path.join(HERE, "oracle.h")]
    if os.path.exists(LIB) and all(os.path.getmtime(d) <= os.path.getmtime(LIB) for d in deps):
        return LIB
    cmd = ["gcc", "-std=c99", "-O2", "-ffp-contract=off", "-fPIC", "-shared", "-Wall", "-o", LIB, *SOURCES, "-lpthread", "-lm"]
    r = subprocess.run(cmd, stdout=subprocess.PIPE, stderr=subprocess.STDOUT, text=True)
    if r.returncode != 0:
        raise RuntimeError("oracle build failed:\n" + r.stdout)
    return LIB


class OrcLeaf(C.Structure):
    _fields_ = [("values", C.c_void_p), ("type", C.c_uint32), ("op", C.c_uint32), ("target", C.c_double)]


def lib():
    global _lib
    if _lib is None:
        build()
        L = C.CDLL(LIB)
        P, u32, u64, dbl = C.c_void_p, C.c_uint32, C.c_uint64, C.c_double
        L.orc_set_threads.argtypes = [u32]
        L.orc_threads.restype = u32
        L.orc_splitmix_draw.argtypes = [u64, u64]
        L.orc_splitmix_draw.restype = u64
        L.orc_fill_splitmix_u32.argtypes = [P, u64, u64, u32, u32, u64]
        L.orc_fill_closed_form.argtypes = [P, P, P, P, u64]
        L.orc_aggregate_global_cpu.argtypes = [P, u32, u64, u32, P, P, P]
        L.orc_aggregate_global_gpu_order.argtypes = [P, u32, u64, P, P, P]
        L.orc_compensated_sum.argtypes = [P, u32, u64]
        L.orc_compensated_sum.restype = dbl
        L.orc_scan_and.argtypes = [P, u32, u64, P, u64]
        L.orc_scan_and.restype = u64
        L.orc_group_dense.argtypes = [P, u32, u64, C.c_int64, u64, u32, P, P, P, P, P, P, P]
        L.orc_group_cpu_reduce.argtypes = [P, u64, u32, P, u64, P, P, P, P, P]
        L.orc_group_cpu_reduce.restype = u64
        L.orc_eval_program.argtypes = [P, u32, P, P, P, P, u64, P]
        L.orc_eval_program.restype = u64
        L.orc_eval_program_scored.argtypes = [P, u32, P, P, P, P, u64, P, P]
        L.orc_eval_program_scored.restype = u64
        L.orc_batch_count_sum.argtypes = [u32, P, P, P, P, P, P, P, u64, P, P]
        L.orc_batch_count_sum.restype = C.c_int
        L.orc_hll_add.argtypes = [P, u64, u32, P]
        L.orc_hll_estimate.argtypes = [P, u64]
        L.orc_hll_estimate.restype = dbl
        L.orc_tdigest_percentile.argtypes = [P, P, u64, dbl]
        L.orc_tdigest_percentile.restype = dbl
        L.orc_sort_rows.argtypes = [P, u32, P, u64, P]
        L.orc_sort_rows.restype = C.c_int
        L.orc_window_rank.argtypes = [P, u32, P, u32, u64, P, P, P, P]
        L.orc_window_rank.restype = C.c_int
        L.orc_join_aggregate.argtypes = [P, P, u64, P, P, u64, u32, P, P]
        L.orc_join_aggregate.restype = C.c_int
        L.orc_fixed_scale.argtypes = [P, u64, P, P]
        L.orc_fixed_scale.restype = C.c_int
        L.orc_fixed_scale_each.argtypes = [P, u64, P]
        L.orc_dense_fixed.argtypes = [P, u64, u32, P, P, P, C.c_int64, u64, P, P, P, P]
        L.orc_dense_fixed.restype = u64
        _lib = L
    return _lib


def _p(a):
    return a.ctypes.data_as(C.c_void_p)


def set_threads(n):
    lib().orc_set_threads(n)


def splitmix_u32(rows, seed, per_row, index, rng):
    out = np.empty(rows, dtype=np.uint32)
    lib().orc_fill_splitmix_u32(_p(out), rows, seed, per_row, index, rng)
    return out


def closed_form(rows):
    cols = [np.empty(rows, dtype=np.uint32) for _ in range(4)]
    lib().orc_fill_closed_form(*[_p(c) for c in cols], rows)
    return cols


_NP_TYPE = {np.dtype(np.uint32): U32, np.dtype(np.int32): I32, np.dtype(np.float32): F32, np.dtype(np.float64): F64,
            np.dtype(np.uint64): U64, np.dtype(np.int64): I64}


def type_of(arr):
    return _NP_TYPE[arr.dtype]


def aggregate_global_cpu(values, tasks=0):
    s, mn, mx = C.c_double(), C.c_double(), C.c_double()
    lib().orc_aggregate_global_cpu(_p(values), type_of(values), len(values), tasks, C.byref(s), C.byref(mn), C.byref(mx))
    return s.value, mn.value, mx.value


def aggregate_global_gpu_order(values):
    s, mn, mx = C.c_double(), C.c_double(), C.c_double()
    lib().orc_aggregate_global_gpu_order(_p(values), type_of(values), len(values), C.byref(s), C.byref(mn), C.byref(mx))
    return s.value, mn.value, mx.value


def compensated_sum(values):
    return lib().orc_compensated_sum(_p(values), type_of(values), len(values))


def scan_and(leaves, rows, want_rows=False):
    """leaves: list of (array, op, target). Returns (count, rows or None)."""
    arr = (OrcLeaf * len(leaves))()
    for i, (a, op, t) in enumerate(leaves):
        arr[i] = OrcLeaf(a.ctypes.data, type_of(a), op, float(t))
    out = None
    cap = 0
    if want_rows:
        out = np.empty(rows, dtype=np.uint32)
        cap = rows
    n = lib().orc_scan_and(arr, len(leaves), rows, _p(out) if out is not None else None, cap)
    return n, (out[:n].copy() if out is not None else None)


def group_dense(key, min_key, groups, funcs, args):
    """funcs: list of codes; args: list of arrays (or None for COUNT). Returns counts, sums, mins, maxs."""
    e = len(funcs)
    counts = np.zeros(groups, dtype=np.uint64)
    sums = np.zeros(groups * e, dtype=np.int64)
    mins = np.zeros(groups * e, dtype=np.int64)
    maxs = np.zeros(groups * e, dtype=np.int64)
    fa = np.array(funcs, dtype=np.uint32)
    keep = [a if a is not None else key for a in args]
    ptrs = (C.c_void_p * e)(*[a.ctypes.data for a in keep])
    types = np.array([type_of(a) for a in keep], dtype=np.uint32)
    lib().orc_group_dense(_p(key), type_of(key), len(key), int(min_key), groups, e, _p(fa), ptrs, _p(types), _p(counts), _p(sums),
                          _p(mins), _p(maxs))
    return counts, sums.reshape(groups, e), mins.reshape(groups, e), maxs.reshape(groups, e)


def group_cpu_reduce(key, args, max_groups):
    e = len(args)
    keys = np.zeros(max_groups, dtype=np.uint32)
    counts = np.zeros(max_groups, dtype=np.uint64)
    sums = np.zeros(max_groups * max(e, 1), dtype=np.float64)
    mins = np.zeros(max_groups * max(e, 1), dtype=np.float64)
    maxs = np.zeros(max_groups * max(e, 1), dtype=np.float64)
    ptrs = (C.c_void_p * max(e, 1))(*[a.ctypes.data for a in args] if e else [None])
    n = lib().orc_group_cpu_reduce(_p(key), len(key), e, ptrs, max_groups, _p(keys), _p(counts), _p(sums), _p(mins), _p(maxs))
    return keys[:n], counts[:n], sums[: n * e].reshape(n, e), mins[: n * e].reshape(n, e), maxs[: n * e].reshape(n, e)


def eval_program(words, consts, str_pool, slot_arrays, slot_types, rows, scores=False):
    """The scan bytecode evaluated per row (orc_eval_program). slot_arrays[s]: the column bound at
    slot s (raw strings: bytes at s, u64 offsets at s + 1), or None. Returns the match mask (uint8)."""
    w = np.ascontiguousarray(words, dtype=np.uint32)
    k = np.ascontiguousarray(consts if len(consts) else [0, 0], dtype=np.uint32)
    sp = np.frombuffer(bytes(str_pool) + b"\0" * 8, dtype=np.uint8).copy()
    keep = [np.ascontiguousarray(a) if a is not None else np.zeros(1, dtype=np.uint64) for a in slot_arrays]
    ptrs = (C.c_void_p * 10)(*[keep[i].ctypes.data if i < len(keep) else None for i in range(10)])
    types = np.zeros(10, dtype=np.uint32)
    types[: len(slot_types)] = slot_types
    mask = np.zeros(max(rows, 1), dtype=np.uint8)
    if scores:
        sc = np.zeros(max(rows, 1), dtype=np.float64)
        lib().orc_eval_program_scored(_p(w), len(w), _p(k), _p(sp), ptrs, _p(types), rows, _p(mask), _p(sc))
        return mask[:rows], sc[:rows]
    lib().orc_eval_program(_p(w), len(w), _p(k), _p(sp), ptrs, _p(types), rows, _p(mask))
    return mask[:rows]


def batch_count_sum(programs, rows):
    """COUNT(*) and the compensated SUM of each program of a batch (orc_batch_count_sum). programs: a list
    of (words, consts, slot_arrays, slot_types, sum_array or None). Returns (counts uint64, sums f64)."""
    n = len(programs)
    keep = []
    words = (C.c_void_p * n)()
    wcount = np.zeros(n, dtype=np.uint32)
    consts = (C.c_void_p * n)()
    slots = (C.c_void_p * (n * 10))()
    types = np.zeros(n * 10, dtype=np.uint32)
    sums = (C.c_void_p * n)()
    stypes = np.zeros(n, dtype=np.uint32)
    for q, (w, k, arrays, st, sarr) in enumerate(programs):
        w = np.ascontiguousarray(w, dtype=np.uint32)
        k = np.ascontiguousarray(k if len(k) else [0, 0], dtype=np.uint32)
        keep += [w, k]
        words[q], wcount[q], consts[q] = w.ctypes.data, len(w), k.ctypes.data
        for s, a in enumerate(arrays[:10]):
            if a is not None:
                a = np.ascontiguousarray(a)
                keep.append(a)
                slots[q * 10 + s] = a.ctypes.data
        types[q * 10: q * 10 + len(st)] = st
        if sarr is not None:
            keep.append(sarr)
            sums[q], stypes[q] = sarr.ctypes.data, type_of(sarr)
    counts = np.zeros(n, dtype=np.uint64)
    out = np.zeros(n, dtype=np.float64)
    if not lib().orc_batch_count_sum(n, words, _p(wcount), consts, slots, _p(types), sums, _p(stypes), rows, _p(counts), _p(out)):
        raise ValueError("a program holds an opcode the batch evaluator does not take")
    return counts, out


def hll_registers(values, p=10):
    v = np.ascontiguousarray(values, dtype=np.float64)
    regs = np.zeros(1 << p, dtype=np.uint32)
    lib().orc_hll_add(_p(v), len(v), p, _p(regs))
    return regs


def hll_estimate(regs):
    r = np.ascontiguousarray(regs, dtype=np.uint32)
    return lib().orc_hll_estimate(_p(r), len(r))


def tdigest_percentile(means, weights, fraction):
    m = np.ascontiguousarray(means, dtype=np.float32)
    w = np.ascontiguousarray(weights, dtype=np.float32)
    return lib().orc_tdigest_percentile(_p(m), _p(w), len(m), fraction)


def sort_rows(keys, desc=None):
    """Row numbers in ORDER BY order: keys compared as F64, DESC per key, ties by position."""
    rows = len(keys[0])
    k = np.ascontiguousarray(np.stack([np.asarray(x).astype(np.float64) for x in keys]))
    d = np.array(desc if desc is not None else [0] * len(keys), dtype=np.uint32)
    out = np.empty(max(rows, 1), dtype=np.uint64)
    if not lib().orc_sort_rows(_p(k), len(keys), _p(d), rows, _p(out)):
        raise MemoryError("orc_sort_rows")
    return out[:rows]


def window_rank(keys, desc=None, partitions=0):
    """ROW_NUMBER / RANK / DENSE_RANK in window order -> (rows, row_number, rank, dense_rank)."""
    rows = len(keys[0])
    k = np.ascontiguousarray(np.stack([np.asarray(x).astype(np.float64) for x in keys]))
    d = np.array(desc if desc is not None else [0] * len(keys), dtype=np.uint32)
    out = np.empty(max(rows, 1), dtype=np.uint64)
    rn, rk, dr = (np.empty(max(rows, 1), dtype=np.uint32) for _ in range(3))
    if not lib().orc_window_rank(_p(k), len(keys), _p(d), partitions, rows, _p(out), _p(rn), _p(rk), _p(dr)):
        raise MemoryError("orc_window_rank")
    return out[:rows], rn[:rows], rk[:rows], dr[:rows]


def gather_column(stored, rows, width=0, base=0):
    """The selected rows of one column (selection_gather.comp:64-78, modes 0/1: dest[i] = source[row i]),
    with the encodings decoded as the scans read them (qe_encoding_shader_width, query_exec.c:1593-1601):
    width 1/2 narrow codes -> base + code, width 3 -> base + row, both in 32-bit arithmetic.
    `stored` is what the column holds (codes for narrow widths, None for a sequence)."""
    r = np.asarray(rows, dtype=np.int64)
    if width == 3:
        return ((base + r) & 0xFFFFFFFF).astype(np.uint32)
    v = np.asarray(stored)[r]
    if width in (1, 2):
        return ((base + v.astype(np.int64)) & 0xFFFFFFFF).astype(np.uint32)
    return v


NO_ROW = 0xFFFFFFFF


def selection_gather(mode, rows, source, positions, count, stride=1, row_offset=0, map_stride=1, word_offset=0, map_offset=0):
    """selection_gather.comp:28-78 for `count` invocations, in 32-bit arithmetic. Modes: 0 an f64 (two
    words) per row, 1 a 32-bit word per row, 2 rows through positions, 3 resolve through a map, 4 resolve
    with an offset. rows/source/positions are u32 word arrays; returns the destination words."""
    rows = np.asarray(rows, dtype=np.uint32)
    src = np.asarray(source, dtype=np.uint32) if source is not None else None
    out = np.zeros(count * (2 if mode == 0 else 1), dtype=np.uint32)
    add = lambda a, b: np.uint32((int(a) + int(b)) & 0xFFFFFFFF)
    for i in range(count):
        if mode == 2:
            index = rows[int(positions[i]) * stride + word_offset]
            out[i] = NO_ROW if index == NO_ROW else add(index, row_offset)
            continue
        index = rows[i * stride + word_offset]
        if mode == 4:
            out[i] = NO_ROW if index == NO_ROW else add(index, row_offset)
        elif mode == 3:
            mapped = NO_ROW if index == NO_ROW else src[int(index) * map_stride]
            out[i] = NO_ROW if mapped == NO_ROW else add(mapped, map_offset)
        else:
            has = index != NO_ROW
            row = int(add(index, row_offset))
            if mode == 0:
                out[2 * i] = src[2 * row] if has else 0
                out[2 * i + 1] = src[2 * row + 1] if has else 0
            else:
                out[i] = src[row] if has else 0
    return out


def gather_strings(values, rows):
    """The selected rows of a string column, as bytes."""
    return [values[int(i)] for i in rows]


def join_aggregate(fact_key, fact_arg, dim_key, dim_group, groups):
    """COUNT(*) and SUM(fact_arg) per group over fact JOIN dim (dim_group 0xffffffff = filtered out)."""
    fk = np.ascontiguousarray(fact_key, dtype=np.uint32)
    fa = np.ascontiguousarray(fact_arg, dtype=np.uint32) if fact_arg is not None else None
    dk = np.ascontiguousarray(dim_key, dtype=np.uint32)
    dg = np.ascontiguousarray(dim_group, dtype=np.uint32)
    counts = np.zeros(groups, dtype=np.uint64)
    sums = np.zeros(groups, dtype=np.int64)
    ok = lib().orc_join_aggregate(_p(fk), _p(fa) if fa is not None else None, len(fk), _p(dk), _p(dg), len(dk), groups,
                                  _p(counts), _p(sums))
    if not ok:
        raise MemoryError("orc_join_aggregate")
    return counts, sums


def fixed_scale(values):
    """qe_values_fixed_point over f64 values -> (scale or -1, largest magnitude)."""
    v = np.ascontiguousarray(values, dtype=np.float64)
    scale = C.c_int32()
    largest = C.c_double()
    lib().orc_fixed_scale(_p(v), len(v), C.byref(scale), C.byref(largest))
    return scale.value, largest.value


def fixed_scale_each(values):
    v = np.ascontiguousarray(values, dtype=np.float64)
    out = np.empty(len(v), dtype=np.int8)
    lib().orc_fixed_scale_each(_p(v), len(v), _p(out))
    return out


def dense_fixed(keys, funcs, args, scales):
    """The dense fixed-point GROUP BY -> dict(keys, first_rows, counts, results[G, E]) of the present groups."""
    k = np.ascontiguousarray(keys, dtype=np.float64)
    e = len(funcs)
    arrs = [np.ascontiguousarray(a, dtype=np.float64) if a is not None else np.zeros(1) for a in args]
    ptrs = (C.c_void_p * e)(*[a.ctypes.data for a in arrs])
    fa = np.array(funcs, dtype=np.uint32)
    sc = np.array(scales, dtype=np.int32)
    lo, hi = (int(k.min()), int(k.max())) if len(k) else (0, 0)
    groups = hi - lo + 1
    ok = np.zeros(groups, dtype=np.int64)
    of = np.zeros(groups, dtype=np.uint64)
    oc = np.zeros(groups, dtype=np.uint64)
    res = np.zeros(groups * e, dtype=np.float64)
    G = lib().orc_dense_fixed(_p(k), len(k), e, _p(fa), ptrs, _p(sc), lo, groups, _p(ok), _p(of), _p(oc), _p(res))
    return {"keys": ok[:G], "first_rows": of[:G], "counts": oc[:G], "results": res[: G * e].reshape(G, e)}
