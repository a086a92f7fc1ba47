"""ctypes bindings of the two native libraries.

libcqlcuda.so is the backend (include/cqlcuda.h); libcqlops.so is the C99 operator layer over it
(include/cqlops.h). Nothing here computes: every result comes from the CUDA kernels. Loading
fails loudly when a library is missing; there is no CPU fallback.
"""
from __future__ import annotations

import ctypes as C
import os

import numpy as np

PKG = os.path.dirname(os.path.abspath(__file__))
LIB_CUDA = os.path.join(PKG, "libcqlcuda.so")
LIB_OPS = os.path.join(PKG, "libcqlops.so")

P, u32, u64, i64, dbl, cstr = C.c_void_p, C.c_uint32, C.c_uint64, C.c_int64, C.c_double, C.c_char_p


class CqlMemoryStats(C.Structure):
    _fields_ = [(n, u64) for n in ("bytes_in_use", "bytes_peak", "alloc_failures", "alloc_retry_successes", "pool_evictions",
                                   "pool_evicted_bytes", "alloc_calls", "unrecovered_alloc_failures")]


class CqlStreamStats(C.Structure):
    _fields_ = [("bytes_copied", u64), ("imports_created", u64), ("import_microseconds", u64), ("staged_bytes", u64),
                ("separate_copy_queue", u32)]


class CqlDict(C.Structure):
    _fields_ = [("count", u32), ("offsets", P), ("bytes", P)]


class CqlColumn(C.Structure):
    _fields_ = [("type", u32), ("width", u32), ("base", u32), ("has_range", u32), ("rows", u64), ("buffer", P),
                ("zone_min", dbl), ("zone_max", dbl), ("offsets", P), ("dict", P), ("zone_map", P), ("zone_map_chunks", u64)]


class CqlHostColumn(C.Structure):
    _fields_ = [("uid", u64), ("generation", u64), ("values", P), ("type", u32), ("has_range", u32), ("zone_min", dbl), ("zone_max", dbl)]


class CqlServeConfig(C.Structure):
    _fields_ = [("workers", u32), ("fuse", u32), ("max_fuse", u32), ("rows_per_thread", u32), ("memory_budget", u64)]


class CqlServeRequest(C.Structure):
    _fields_ = [("kind", u32), ("table", u32), ("program", P), ("sum_column", C.c_int32), ("column_count", u32), ("columns", u32 * 4),
                ("expr_count", u32), ("funcs", u32 * 8), ("args", C.c_int32 * 8), ("max_groups", u64), ("out_counts", P),
                ("out_sums", P), ("out_mins", P), ("out_maxs", P), ("call", P), ("ctx", P), ("footprint", u64), ("count", u64),
                ("min_key", i64), ("sum", dbl * 4), ("min", dbl * 4), ("max", dbl * 4), ("status", C.c_int32), ("fused", u32),
                ("submit_ns", u64), ("start_ns", u64), ("done_ns", u64), ("error", C.c_char * 128), ("next", P)]


class CqlServeStats(C.Structure):
    _fields_ = [(n, u64) for n in ("submitted", "completed", "failed", "scans", "fused_requests", "max_fused", "in_flight_bytes",
                                   "peak_in_flight_bytes", "memory_budget", "admission_waits", "merged_requests")]


RESIDENT_ALLOC = C.CFUNCTYPE(C.c_void_p, C.c_void_p, u64)
RESIDENT_COPY = C.CFUNCTYPE(C.c_int, C.c_void_p, C.c_void_p, C.c_void_p, u64)
RESIDENT_RELEASE = C.CFUNCTYPE(None, C.c_void_p, C.c_void_p)
RESIDENT_MEMORY = C.CFUNCTYPE(u64, C.c_void_p)


class CqlResidentOps(C.Structure):
    _fields_ = [("alloc", RESIDENT_ALLOC), ("copy", RESIDENT_COPY), ("release", RESIDENT_RELEASE), ("total_memory", RESIDENT_MEMORY),
                ("free_memory", RESIDENT_MEMORY), ("ctx", P)]


class CqlResidentStats(C.Structure):
    _fields_ = [(n, u64) for n in ("hit_bytes", "miss_bytes", "evicted_bytes", "bytes_in_use", "entries", "budget_bytes")]


class CqlLeaf(C.Structure):
    _fields_ = [("column", u32), ("op", u32), ("target", dbl)]


MAX_WORDS, MAX_CONSTS, MAX_STR_POOL, MAX_BINDINGS = 4096, 256, 65536, 10


class CqlProgram(C.Structure):
    _fields_ = [("words", u32 * MAX_WORDS), ("word_count", u32), ("consts", u32 * (2 * MAX_CONSTS)), ("const_count", u32),
                ("str_pool", C.c_uint8 * MAX_STR_POOL), ("str_pool_size", u32), ("binding_count", u32),
                ("binding_column", u32 * MAX_BINDINGS), ("binding_type", u32 * MAX_BINDINGS), ("binding_slot", u32 * MAX_BINDINGS),
                ("binding_dict", u32 * MAX_BINDINGS), ("next_slot", u32), ("requires_cpu_scan", u32), ("has_score_output", u32),
                ("error", C.c_char * 128)]


class CqlJoinAgg(C.Structure):
    _fields_ = [("fact_key", P), ("expr_count", u32), ("funcs", P), ("fact_args", P), ("dim_args", P), ("dim_keys", P),
                ("dim_table_rows", u64), ("dim_rows", P), ("dim_count", u64), ("group_count", u32), ("dim_group_values", P),
                ("strategy", u32), ("dim_key_column", P), ("dim_group_column", P)]


class CqlServeJoin(C.Structure):
    _fields_ = [("query", CqlJoinAgg), ("max_groups", u64), ("out_group_dim_row", P), ("out_results", P), ("groups", u64),
                ("strategy", u32)]


class CqlServeSort(C.Structure):
    _fields_ = [("columns", P), ("column_count", u32), ("leaves", P), ("leaf_count", u32), ("sort_column", u32), ("desc", u32),
                ("max_rows", u64), ("limit", u64), ("out_rows", P), ("count", u64)]


class CqlFusedAgg(C.Structure):
    _fields_ = [("column_count", u32), ("slots", u32 * 4), ("coltypes", u32 * 4), ("grouped", u32), ("key_count", u32),
                ("key_slots", u32 * 3), ("key_types", u32 * 3), ("key_ranges", u32 * 3), ("group_count", u32)]


# (name, restype, argtypes) of every entry point include/cqlcuda.h declares
CUDA_API = [
    ("cqlcuda_init", C.c_int, []),
    ("cqlcuda_release", None, []),
    ("cqlcuda_wait", None, []),
    ("cqlcuda_get_executed_kernel_time_microseconds", u64, []),
    ("cqlcuda_device_total_memory", u64, []),
    ("cqlcuda_device_free_memory", u64, []),
    ("cqlcuda_device_max_storage_buffer_range", u64, []),
    ("cqlcuda_device_lost", C.c_int, []),
    ("cqlcuda_pool_begin_epoch", None, []),
    ("cqlcuda_pool_evict", u64, [u64]),
    ("cqlcuda_memory_stats", CqlMemoryStats, []),
    ("cqlcuda_sm_count", u32, []),
    ("cqlcuda_buffer_alloc", P, [u64, u32, P]),
    ("cqlcuda_buffer_alloc_pooled", P, [cstr, u64, u64, u32, P]),
    ("cqlcuda_buffer_import_host_readonly", P, [P, u64]),
    ("cqlcuda_buffer_import_host_readonly_pooled", P, [cstr, u64, P, u64]),
    ("cqlcuda_buffer_release", None, [P]),
    ("cqlcuda_buffer_write", None, [P, P, u64]),
    ("cqlcuda_buffer_read", None, [P, P, u64]),
    ("cqlcuda_buffer_size", u64, [P]),
    ("cqlcuda_buffer_device_pointer", P, [P]),
    ("cqlcuda_kernel_alloc", P, [cstr, u64]),
    ("cqlcuda_kernel_alloc_from_image", P, [cstr, u64, P, u64]),
    ("cqlcuda_kernel_alloc_from_image_spec", P, [cstr, u64, P, u64, P, u32]),
    ("cqlcuda_generated_kernel_stats", None, [P, P]),
    ("cqlcuda_set_generated_kernel_cap", None, [u32]),
    ("cqlcuda_kernel_release", None, [P]),
    ("cqlcuda_kernel_execute", None, [P, u32, u32]),
    ("cqlcuda_kernel_set_arg_buffer", None, [P, u32, P]),
    ("cqlcuda_kernel_set_arg_u64", None, [P, u32, u64]),
    ("cqlcuda_kernel_set_arg_buffer_range", None, [P, u32, P, u64, u64]),
    ("cqlcuda_batch_begin", P, [u64, u64]),
    ("cqlcuda_batch_begin_graph", P, [u64, u64, u64]),
    ("cqlcuda_graph_stats", None, [P, P, P]),
    ("cqlcuda_graph_enable", None, [C.c_int]),
    ("cqlcuda_batch_buffer_write", None, [P, P, P, u64]),
    ("cqlcuda_batch_buffer_zero", None, [P, P, u64]),
    ("cqlcuda_batch_buffer_fill", None, [P, P, u64, u32]),
    ("cqlcuda_batch_kernel_execute", None, [P, P, u32, u32]),
    ("cqlcuda_batch_buffer_read", None, [P, P, P, u64]),
    ("cqlcuda_batch_buffer_read_at", None, [P, P, u64, P, u64]),
    ("cqlcuda_batch_fill_range", None, [P, P, u64, u64, u32]),
    ("cqlcuda_batch_end", C.c_int, [P]),
    ("cqlcuda_stream_alloc", P, [u32]),
    ("cqlcuda_stream_release", None, [P]),
    ("cqlcuda_stream_slot_begin", C.c_int, [P, u32, u64, u64]),
    ("cqlcuda_stream_copy", C.c_int, [P, u32, P, P, u64]),
    ("cqlcuda_stream_zero", None, [P, u32, P, u64]),
    ("cqlcuda_stream_fill", None, [P, u32, P, u64, u32]),
    ("cqlcuda_stream_dispatch", None, [P, u32, P, u32, u32]),
    ("cqlcuda_stream_read", None, [P, u32, P, P, u64]),
    ("cqlcuda_stream_submit", C.c_int, [P, u32]),
    ("cqlcuda_stream_wait", C.c_int, [P, u32]),
    ("cqlcuda_stream_get_stats", CqlStreamStats, [P]),
    ("cqlcuda_set_fault_alloc_at", None, [u64]),
    ("cqlcuda_set_evict_hook", None, [P]),
    ("cqlcuda_kernel_profile_enable", None, [C.c_int]),
    ("cqlcuda_kernel_profile_reset", None, []),
    ("cqlcuda_kernel_profile_entry", C.c_int, [u32, P, P, P]),
    ("cqlcuda_host_profile", None, [P, P, P, P]),
    ("cqlcuda_kernel_launch_count", u32, []),
    ("cqlcuda_last_error", cstr, []),
    ("cqlcuda_clear_error", None, []),
    ("cqlcuda_set_wait_timeout_ms", None, [u32]),
    ("cqlcuda_set_module_cache_dir", None, [cstr]),
    ("cqlcuda_set_fail_compile_every", None, [u32]),
    ("cqlcuda_last_compile_log", cstr, []),
    ("cqlcuda_compile_check", C.c_int, [cstr, u64]),
    ("cqlcuda_compact_slots_noalloc", C.c_int, [P, P, u32, P, P, P, P, P]),
    ("cqlcuda_thread_lane_begin", C.c_int, [cstr]),
    ("cqlcuda_thread_lane_end", None, []),
    ("cqlcuda_fill_splitmix_u32", C.c_int, [P, u64, u64, u32, u32, u64]),
    ("cqlcuda_fill_sequence_u32", C.c_int, [P, u64, u32]),
    ("cqlcuda_fill_affine_u32", C.c_int, [P, u64, u64, u64, u64]),
    ("cqlcuda_host_alloc", P, [u64]),
    ("cqlcuda_host_free", None, [P]),
    ("cqlcuda_buffer_alloc_host_mapped", P, [u64, P]),
    ("cqlcuda_persistent_create", P, [P, cstr]),
    ("cqlcuda_persistent_launch", C.c_int, [P, u32, P, u64]),
    ("cqlcuda_persistent_running", C.c_int, [P]),
    ("cqlcuda_persistent_copy", C.c_int, [P, P, u64, P, u64]),
    ("cqlcuda_persistent_destroy", C.c_int, [P, u32]),
    ("cqlcuda_persistent_ctas", u32, [P]),
    ("cqlcuda_flush_l2", C.c_int, [u64]),
    ("cqlcuda_timer_begin", None, []),
    ("cqlcuda_timer_end_ms", dbl, []),
]

OPS_API = [
    ("cqlops_aggregate_global", C.c_int, [P, u32, P, P, P]),
    ("cqlops_scan_simple", C.c_int, [P, u32, P, u32, P, P, u64]),
    ("cqlops_scan_simple_select", C.c_int, [P, u32, P, u32, P, P]),
    ("cqlops_group_dense", C.c_int, [P, u64, u32, P, P, u64, P, P, P, P, P, P]),
    ("cqlops_last_launches", u32, []),
    ("cqlops_last_error", cstr, []),
    ("cqlops_program_build", C.c_int, [cstr, P, P, u32, P]),
    ("cqlops_program_bind", C.c_int, [P, P, u32]),
    ("cqlops_program_max_stack_depth", u32, [P]),
    ("cqlops_program_simple_leaves", u32, [P, P, u32]),
    ("cqlops_program_source", C.c_int, [P, u32, P, P, u64, P]),
    ("cqlops_scan_filter", C.c_int, [P, P, u32, P, P, u64, P]),
    ("cqlops_scan_filter_scored", C.c_int, [P, P, P, P, P, u64]),
    ("cqlops_fused_filter_aggregate", C.c_int, [P, P, P, u32, P, P, P, P]),
    ("cqlops_fused_filter_group", C.c_int, [P, P, P, u32, P, u32, u64, P, P, P, P, P, P, P, P]),
    ("cqlops_group_hash", C.c_int, [P, u32, u32, P, P, P, u64, u32, u64, P, P, P, P, P]),
    ("cqlops_hash_join", C.c_int, [P, P, C.c_int, u64, P, P, u64]),
    ("cqlops_join_aggregate", C.c_int, [P, u64, P, P, P, P]),
    ("cqlops_sort_rows", C.c_int, [P, u32, P, P, u64, P, u64]),
    ("cqlops_window_rank", C.c_int, [P, u32, P, u32, P, u64, P, P, P, P, u64]),
    ("cqlops_having", C.c_int, [cstr, P, u32, P, u32, u64, P]),
    ("cqlops_having_source", C.c_int, [cstr, u32, P, u64, P]),
    ("cqlops_gather_rows", C.c_int, [P, u32, P, P, u64, P]),
    ("cqlops_gather_strings", C.c_int, [P, P, P, u64, P, P, u64, P]),
    ("cqlops_fixed_scale", C.c_int, [P, P, u64, P, P]),
    ("cqlops_zone_map_build", C.c_int, [P, P, u64]),
    ("cqlops_batch_last_form", u32, []),
    ("cqlops_batch_tuner_reset", None, []),
    ("cqlops_batch_filter_aggregate", C.c_int, [P, u32, P, u32, P, u32, P, P, P]),
    ("cqlops_batch_source", C.c_int, [P, u32, P, u32, P, u32, P, u64, P, P]),
    ("cqlops_batch_cube_source", C.c_int, [P, u32, P, u32, P, u32, P, u64, P, P]),
    ("cqlops_batch_catalog_create", P, []),
    ("cqlops_batch_catalog_destroy", None, [P]),
    ("cqlops_batch_catalog_shapes", u32, [P]),
    ("cqlops_batch_filter_aggregate_cat", C.c_int, [P, P, u32, P, u32, P, u32, P, P, P]),
    ("cqlops_batch_prepare", C.c_int, [P, P, u32, P, u32, P, u32]),
    ("cqlops_batch_persist_create", P, [P, P, u32, u32, u32]),
    ("cqlops_batch_persist_run", C.c_int, [P, P, u32, P, P, P]),
    ("cqlops_batch_persist_stats", None, [P, P, P, P]),
    ("cqlops_batch_persist_destroy", C.c_int, [P]),
    ("cqlops_batch_persist_ctas", u32, [P]),
    ("cqlops_resident_create", P, [u64, P]),
    ("cqlops_resident_destroy", None, [P]),
    ("cqlops_resident_acquire", P, [P, u64, u64, P, u64, u64, u32, P]),
    ("cqlops_resident_release", None, [P, P]),
    ("cqlops_resident_evict", u64, [P, u64]),
    ("cqlops_resident_clear", None, [P]),
    ("cqlops_resident_stats", CqlResidentStats, [P]),
    ("cqlops_aggregate_global_streamed", C.c_int, [P, u64, u64, P, u32, u64, u64, P, P, P, P]),
    ("cqlops_aggregate_global_accumulate", C.c_int, [P, u32, P, P, P]),
    ("cqlops_scan_simple_streamed", C.c_int, [P, P, u32, u64, P, u32, u64, P, P, u64, P]),
    ("cqlops_group_dense_streamed", C.c_int, [P, P, u64, u32, P, P, u64, u64, P, P, P, P, P, P, P]),
    ("cqlops_join_aggregate_streamed", C.c_int, [P, P, P, P, u64, u64, u64, P, P, P, P, P]),
    ("cqlserve_create", P, [P]),
    ("cqlserve_destroy", None, [P]),
    ("cqlserve_add_table", C.c_int, [P, P, u32]),
    ("cqlserve_prepare", C.c_int, [P, u32, P, u32, P]),
    ("cqlserve_submit", C.c_int, [P, P]),
    ("cqlserve_wait", C.c_int, [P, P, u32]),
    ("cqlserve_drain", None, [P]),
    ("cqlserve_stats", CqlServeStats, [P]),
    ("cqlserve_join_call", C.c_int, [P]),
    ("cqlserve_sort_call", C.c_int, [P]),
    ("cqlops_scan_ranges", u64, [P, u32, P, u32, P, u64, P, P, P]),
    ("cqlops_group_dense_fixed", C.c_int, [P, u32, P, P, P, u64, u64, P, P, P, P, P, P]),
    ("cqlops_hll_estimate", dbl, [P, u64]),
    ("cqlops_group_hash_registers", u64, [P, u64]),
    ("cqlops_tdigest_percentile", dbl, [P, P, u64, dbl]),
]

_cuda = None
_ops = None


def _bind(lib, api):
    for name, res, args in api:
        f = getattr(lib, name)
        f.restype = res
        f.argtypes = args


def load_cuda():
    global _cuda
    if _cuda is None:
        if not os.path.exists(LIB_CUDA):
            raise RuntimeError(f"{LIB_CUDA} is not built: run computeql_gb300.build.build() (or __graft_entry__.build())")
        lib = C.CDLL(LIB_CUDA, mode=C.RTLD_GLOBAL)
        _bind(lib, CUDA_API)
        _cuda = lib
    return _cuda


def load_ops():
    global _ops
    if _ops is None:
        load_cuda()
        if not os.path.exists(LIB_OPS):
            raise RuntimeError(f"{LIB_OPS} is not built")
        lib = C.CDLL(LIB_OPS)
        _bind(lib, OPS_API)
        _ops = lib
    return _ops


class CudaError(RuntimeError):
    pass


def last_error():
    msgs = []
    if _ops is not None:
        e = _ops.cqlops_last_error()
        if e:
            msgs.append(e.decode())
    e = load_cuda().cqlcuda_last_error()
    if e:
        msgs.append(e.decode())
    return "; ".join(msgs)


def init():
    lib = load_cuda()
    if not lib.cqlcuda_init():
        raise CudaError("cqlcuda_init failed: " + last_error())
    return lib


def ptr(a):
    return C.c_void_p(a.ctypes.data)
