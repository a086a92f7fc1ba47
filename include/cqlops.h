/*
 * cqlops.h - C99 operator layer over the cqlcuda C ABI.
 *
 * Each function drives the backend the way the reference's operator layer drives its GPU
 * (src/query_exec/query_exec.c): the same kernels by name, the same bindings and push-constant
 * words, the same host folds. Columns are passed as plain descriptors instead of CQL_Column, and a
 * column is held whole in device memory (one "chunk"), because GB300's HBM holds the configured
 * tables resident; the reference streams 16M-row chunks through 2 GB buffers.
 *
 * Return values follow the reference operators: 1 on success, 0 when the request is not one the
 * path handles or the GPU work failed (nothing is written to the outputs then, and
 * cqlcuda_last_error() says why).
 */
#ifndef CQLOPS_H
#define CQLOPS_H

#include <stdint.h>
#include "cqlcuda.h"

#ifdef __cplusplus
extern "C" {
#endif

/* CQL_ColumnType values (src/cql/cql.h:79-95). */
enum
{
  CQLOPS_TYPE_U32 = 1,
  CQLOPS_TYPE_U64 = 2,
  CQLOPS_TYPE_F32 = 3,
  CQLOPS_TYPE_F64 = 4,
  CQLOPS_TYPE_STRING8 = 5,
  CQLOPS_TYPE_BOOL = 6,
  CQLOPS_TYPE_I32 = 7,
  CQLOPS_TYPE_I64 = 8,
};

/* Aggregate function codes (src/query_exec/query_exec.h:902-909). */
enum
{
  CQLOPS_FUNC_COUNT = 0,
  CQLOPS_FUNC_SUM = 1,
  CQLOPS_FUNC_AVG = 2,
  CQLOPS_FUNC_MIN = 3,
  CQLOPS_FUNC_MAX = 4,
  CQLOPS_FUNC_APPROX_COUNT_DISTINCT = 5,
  CQLOPS_FUNC_APPROX_PERCENTILE = 6,
};

/* Comparison operators of scan_simple leaves (src/gpu/vulkan/shaders/scan_simple.comp:15-19). */
enum
{
  CQLOPS_CMP_EQ = 0,
  CQLOPS_CMP_LT = 1,
  CQLOPS_CMP_LE = 2,
  CQLOPS_CMP_GT = 3,
  CQLOPS_CMP_GE = 4,
};

/* A string dictionary: value i is bytes[offsets[i] .. offsets[i+1]) (CQL_StringDict, src/cql/cql.h:146-153). */
typedef struct CqlDict
{
  uint32_t count;
  const uint32_t* offsets;
  const char* bytes;
} CqlDict;

/* A device-resident column. `width` is the encoding the kernels are told
   (qe_encoding_shader_width, query_exec.c:1593-1601): 0 = stored as is, 1/2 = narrow codes of that
   many bytes with value = base + code, 3 = a sequence (value = base + row number, nothing stored).
   zone_min/zone_max stand in for the zone map range (qe_column_range_from_zone_map).
   A STRING8 column holds its bytes in `buffer` and (rows + 1) u64 offsets in `offsets`; with a
   dictionary, `buffer` holds the u32 codes instead and `dict` the values (host side).
   zone_map (optional, host memory) holds the column's zone map: (min, max) as f64 for each chunk of
   CQLOPS_ZONEMAP_CHUNK_ROWS rows, zone_map_chunks of them, then one more pair: the largest chunk min
   and the smallest chunk max (cqlops_zone_map_build fills it); scans prune chunks with it. A
   sequence column needs none. */
#define CQLOPS_ZONEMAP_CHUNK_ROWS 8192
/* The most rows one operator call takes: row numbers and counts are 32-bit words in the kernels'
   push constants. Every cqlops_* operator refuses a larger column (returns 0, cqlops_last_error()
   says why) before any device work. */
#define CQLOPS_MAX_ROWS 0xfffffffeull

typedef struct CqlColumn
{
  uint32_t type;
  uint32_t width;
  uint32_t base;
  uint32_t has_range;
  uint64_t rows;
  CqlBuffer* buffer;
  double zone_min;
  double zone_max;
  CqlBuffer* offsets;
  const CqlDict* dict;
  const double* zone_map;
  uint64_t zone_map_chunks;
} CqlColumn;

/* One comparison `column op target` of an AND-only filter (the leaves qe_scan_filter_selected
   hands to scan_simple, query_exec.c:2566-2680). */
typedef struct CqlLeaf
{
  uint32_t column;    /* index into the column array */
  uint32_t op;        /* CQLOPS_CMP_* */
  double target;
} CqlLeaf;

/* ---- WHERE bytecode (QE_BytecodeProgram, src/query_exec/query_exec.h:96-126) ---- */
#define CQLOPS_MAX_WORDS 4096
#define CQLOPS_MAX_CONSTS 256
#define CQLOPS_MAX_STR_POOL 65536
#define CQLOPS_MAX_BINDINGS 10

typedef struct CqlProgram
{
  uint32_t words[CQLOPS_MAX_WORDS];
  uint32_t word_count;
  uint32_t consts[CQLOPS_MAX_CONSTS * 2];     /* f64 constants as (lo, hi) words */
  uint32_t const_count;
  uint8_t str_pool[CQLOPS_MAX_STR_POOL];
  uint32_t str_pool_size;
  uint32_t binding_count;
  uint32_t binding_column[CQLOPS_MAX_BINDINGS];  /* index into the caller's column array */
  uint32_t binding_type[CQLOPS_MAX_BINDINGS];    /* the type it is read as (U32 for dictionary codes) */
  uint32_t binding_slot[CQLOPS_MAX_BINDINGS];    /* first column slot: binding 6 + slot */
  uint32_t binding_dict[CQLOPS_MAX_BINDINGS];    /* 1 when the binding is dictionary codes */
  uint32_t next_slot;
  uint32_t requires_cpu_scan;
  uint32_t has_score_output;                     /* 1: a SIMILARITY score, 2: an EDIT_DISTANCE score per matching row */
  char error[128];
} CqlProgram;

/* Compiles a WHERE condition given as an s-expression over the named columns (qe_bytecode_program_build,
   query_exec.c:510-530; grammar in computeql_gb300/host/cql_program.c). An empty condition is TRUE.
   Returns 0 and sets prog->error on a malformed or unsupported condition. */
int cqlops_program_build(const char* where, const CqlColumn* columns, const char* const* names, uint32_t column_count, CqlProgram* prog);
/* Binds one more column to the program (the fused aggregates' argument and key columns); returns its slot or -1. */
int cqlops_program_bind(CqlProgram* prog, const CqlColumn* columns, uint32_t column_index);
/* qe_bytecode_program_max_stack_depth (query_exec.c:552-612). */
uint32_t cqlops_program_max_stack_depth(const CqlProgram* prog);
/* The leaves of an AND-only tree of numeric comparisons with literals, the shape scan_simple runs;
   0 when the program has another shape. */
uint32_t cqlops_program_simple_leaves(const CqlProgram* prog, CqlLeaf* out, uint32_t cap);

/* ---- per-query kernels (qk_* of src/query_exec/query_kernel.h:198-240, emitted as CUDA C++) ---- */
enum
{
  CQLOPS_KERNEL_SCAN = 0,        /* scan_filter.comp's bindings: matching rows compacted */
  CQLOPS_KERNEL_FUSED_AGG = 1,   /* WHERE + COUNT and SUM/MIN/MAX per column, partials per workgroup */
  CQLOPS_KERNEL_FUSED_GROUP = 2, /* WHERE + GROUP BY up to 3 small-range keys */
};

/* QK_FusedAgg (src/query_exec/query_kernel.h:171-196). */
typedef struct CqlFusedAgg
{
  uint32_t column_count;
  uint32_t slots[4];
  uint32_t coltypes[4];
  uint32_t grouped;
  uint32_t key_count;
  uint32_t key_slots[3];
  uint32_t key_types[3];
  uint32_t key_ranges[3];
  uint32_t group_count;
} CqlFusedAgg;

/* The CUDA C++ source of a program's kernel of the given kind (qk_scan_source_build,
   query_kernel.c:971-1672). Writes at most cap bytes (NUL-terminated) and the length to out_len.
   Returns 0 when the program has an opcode the generated kernel does not take (the reason is
   written to out then). */
int cqlops_program_source(const CqlProgram* prog, uint32_t kind, const CqlFusedAgg* fuse, char* out, uint64_t cap, uint64_t* out_len);

/* Scan strategies of cqlops_scan_filter (the kernel choice cascade of qe_scan_filter_selected,
   query_exec.c:2566-2680). */
enum
{
  CQLOPS_SCAN_AUTO = 0,         /* scan_simple for numeric AND leaves, else the per-query kernel, else the interpreter */
  CQLOPS_SCAN_INTERPRETER = 1,  /* scan_filter: the bytecode interpreter */
  CQLOPS_SCAN_GENERATED = 2,    /* the per-query NVRTC kernel only */
  CQLOPS_SCAN_SIMPLE = 3,       /* scan_simple only */
};

/* Runs a WHERE program over the columns: the count of matching rows and, when out_rows is not NULL,
   up to out_capacity of them in ascending order. out_strategy (may be NULL) receives the strategy
   that ran. */
int cqlops_scan_filter(const CqlProgram* prog, const CqlColumn* columns, uint32_t strategy, uint64_t* out_count, uint32_t* out_rows,
                       uint64_t out_capacity, uint32_t* out_strategy);

/* cqlops_scan_filter for a program with a fuzzy comparison (has_score_output): it runs on the interpreter
   (scan_filter, as in the reference) and writes, next to each of the first out_capacity matching rows in
   ascending order, the row's score - the trigram similarity as the f32 the kernel reports, or the edit
   distance (scan_filter.comp:510-527). Programs without a fuzzy comparison get score 0. */
int cqlops_scan_filter_scored(const CqlProgram* prog, const CqlColumn* columns, uint64_t* out_count, uint32_t* out_rows, double* out_scores,
                              uint64_t out_capacity);

/* WHERE + COUNT(*) and SUM/MIN/MAX of up to 4 numeric columns in one pass (qe_fused_filter_aggregate,
   query_exec.c:9888-10254). agg_columns index the column array. Partials are folded in workgroup order. */
int cqlops_fused_filter_aggregate(const CqlProgram* prog, const CqlColumn* columns, const uint32_t* agg_columns, uint32_t agg_count,
                                  double* out_count, double* out_sum, double* out_min, double* out_max);

/* WHERE + GROUP BY up to 3 small-range whole-number (or dictionary-coded) keys with COUNT and
   SUM/MIN/MAX of up to 4 U32/I32 columns (qe_fused_filter_group_aggregate, query_exec.c:9442-9886).
   Per group g (the keys as digits, key 0 most significant): out_counts[g], out_min_row[g] (the
   smallest matching row), out_sums/out_mins/out_maxs[g*agg_count + c]. out_group_total receives the
   number of groups (the product of the key ranges); the arrays must hold max_groups groups. */
int cqlops_fused_filter_group(const CqlProgram* prog, const CqlColumn* columns, const uint32_t* key_columns, uint32_t key_count,
                              const uint32_t* agg_columns, uint32_t agg_count, uint64_t max_groups, uint64_t* out_group_total,
                              int64_t* out_key_min, uint32_t* out_key_range, uint64_t* out_counts, uint64_t* out_min_row, int64_t* out_sums,
                              int64_t* out_mins, int64_t* out_maxs);

/* SUM/MIN/MAX of up to 4 whole columns (qe_aggregate_global_streamed, query_exec.c:8842-9112, one
   chunk). Partials are folded in workgroup order. Sequence columns are summed in closed form. */
int cqlops_aggregate_global(const CqlColumn* columns, uint32_t column_count, double* out_sum, double* out_min, double* out_max);
/* cqlops_aggregate_global adding every workgroup partial, in workgroup order, into running totals the
   caller carries from chunk to chunk (qe_agg_stream_retire, query_exec.c:8812-8841: one column_sum over
   every partial of every chunk; start them at 0, +F64_MAX and -F64_MAX). */
int cqlops_aggregate_global_accumulate(const CqlColumn* columns, uint32_t column_count, double* io_sum, double* io_min, double* io_max);

/* AND of up to 8 numeric comparisons over up to 10 columns with scan_simple
   (qe_scan_filter_selected, query_exec.c:2495-3276). Writes the match count; when out_rows is not
   NULL and out_capacity > 0 also up to out_capacity matching row numbers in ascending order (the kernel
   writes a bitmap of the rows, which becomes the ascending list on the device).
   When out_rows is NULL the kernel runs count-only. */
int cqlops_scan_simple(const CqlColumn* columns, uint32_t column_count, const CqlLeaf* leaves, uint32_t leaf_count,
                       uint64_t* out_count, uint32_t* out_rows, uint64_t out_capacity);

/* cqlops_scan_simple with the matching rows kept on the device: up to size / 4 of them, ascending, written
   into out_selection (a device buffer) in the same batch as the scan, for the operators that take a
   selection (sort, window, gather, fixed-point GROUP BY) - the selection qe_scan_filter_selected keeps on
   the device for the next operator (keep_on_device, query_exec.c:2793, 3156-3164). Writes the match count. */
int cqlops_scan_simple_select(const CqlColumn* columns, uint32_t column_count, const CqlLeaf* leaves, uint32_t leaf_count,
                              CqlBuffer* out_selection, uint64_t* out_count);

/* GROUP BY one small-range whole-number key (or a dictionary string column, by its codes) with
   COUNT/SUM/AVG/MIN/MAX over whole-number columns (qe_dense_stream_core, query_exec.c:7632-7983, one
   chunk). funcs[e]/arg_cols[e] describe
   expression e (arg_cols[e] is ignored for COUNT). Outputs, per group g = key - min_key:
   out_counts[g], out_sums[g*exprs+e] (64-bit two's complement), out_mins/out_maxs[g*exprs+e]
   (INT32_MAX / INT32_MIN when the group has no rows). out_group_count receives the group count;
   the output arrays must hold max_groups entries (times exprs). */
int cqlops_group_dense(const CqlColumn* key, uint64_t rows, uint32_t expr_count, const uint32_t* funcs, const CqlColumn* const* arg_cols,
                       uint64_t max_groups, uint64_t* out_group_count, int64_t* out_min_key, uint64_t* out_counts, int64_t* out_sums,
                       int64_t* out_mins, int64_t* out_maxs);

/* Hash GROUP BY of up to 4 keys (numeric, widened to f64, or raw strings) with up to 8 aggregates:
   COUNT/SUM/AVG/MIN/MAX, APPROX_COUNT_DISTINCT (HyperLogLog, precision 10) and APPROX_PERCENTILE
   (t-digest, params[e] is the fraction) - qe_aggregate_impl's GPU hash path,
   src/query_exec/query_exec.c:10258-12300. group_hint > 0 sizes the table for that many groups.
   path: 0 automatic, 1 member lists + aggregate_reduce, 2 the fixed-point atomic reduce, 3 one whole-number
   key of at most 64 values with COUNT/SUM/AVG/MIN/MAX over f32/f64 columns: the sums from the batched
   shared scan (exact scaled-integer sums), MIN/MAX and each group's first row from one more pass (groups in
   key order, each represented by its first row; automatic takes it when it
   applies and some argument is not a decimal of at most 6 places, which path 2 finalizes as the
   reference does). Per dense group g: out_repr_row[g] (a row of the group), out_counts[g],
   out_results[g*expr_count + e]. out_path receives the path taken (1, 2 or 3). */
int cqlops_group_hash(const CqlColumn* keys, uint32_t key_count, uint32_t expr_count, const uint32_t* funcs, const CqlColumn* const* args,
                      const double* params, uint64_t group_hint, uint32_t path, uint64_t max_groups, uint64_t* out_group_count,
                      uint64_t* out_repr_row, uint64_t* out_counts, double* out_results, uint32_t* out_path);
/* The HyperLogLog registers behind the calling thread's last cqlops_group_hash: per dense group g, per
   APPROX_COUNT_DISTINCT expression h (in expression order), 2^10 registers at ((g * hll_exprs + h) << 10),
   each the largest rho seen (hll_add, aggregate_reduce.comp:66-92). Copies up to `capacity` words into
   `out` (may be NULL) and returns the word count (0 when that call had no APPROX_COUNT_DISTINCT or
   failed). */
uint64_t cqlops_group_hash_registers(uint32_t* out, uint64_t capacity);
/* qe_hll_estimate_cardinality (query_exec.c:6711-6737) over m registers. */
double cqlops_hll_estimate(const uint32_t* registers, uint64_t m);
/* qe_tdigest_estimate_percentile (query_exec.c:6748-6790); sorts the centroids in place. */
double cqlops_tdigest_percentile(float* means, float* weights, uint64_t count, double fraction);

/* Equi-join of two key columns (numeric, compared as f64 values, or raw strings) - qe_hash_join_impl's
   GPU path, src/query_exec/query_exec.c:14541-15358: the build side hashed into buckets (a power of
   two >= its rows), bucket lists by prefix sum and scatter, every probe row emitting its
   (probe row, build row) pairs; a LEFT join also emits (probe row, 0xffffffff) for an unmatched row.
   hint_pairs > 0 sizes the output for that many pairs. Writes the pair count and up to
   out_capacity pairs, sorted, as (probe, build) u32 pairs. */
int cqlops_hash_join(const CqlColumn* build_key, const CqlColumn* probe_key, int left_join, uint64_t hint_pairs, uint64_t* out_count,
                     uint32_t* out_pairs, uint64_t out_capacity);

/* A join of a fact table to a dim table aggregated by dim columns (qe_aggregate_join_pushdown,
   query_exec.c:8442-8776). */
typedef struct CqlJoinAgg
{
  const CqlColumn* fact_key;          /* device, U32 or I32 */
  uint32_t expr_count;
  const uint32_t* funcs;              /* COUNT/SUM/AVG/MIN/MAX */
  const CqlColumn* const* fact_args;  /* per expression: a fact column (device), or NULL */
  const double* const* dim_args;      /* per expression: a dim column as f64 (host), or NULL; may itself be NULL */
  const uint32_t* dim_keys;           /* host, the dim key column (dim_table_rows entries, same type as fact_key) */
  uint64_t dim_table_rows;
  const uint64_t* dim_rows;           /* the dim rows that pass the dim-side filter, NULL = all */
  uint64_t dim_count;
  uint32_t group_count;               /* GROUP BY dim columns */
  const double* const* dim_group_values; /* host, f64 per dim row */
  uint32_t strategy;                  /* 0 automatic, 1 dense over the fact key's range, 2 probe a hash table of the dim keys,
                                         3 a lookup table over the fact key's range (unique dim keys, at most one
                                         whole-number GROUP BY value spanning < 65536, no dim-side aggregates, a key
                                         range up to 2^24; automatic picks it for ranges above 65536 when it applies) */
  /* Optional: the dim table resident on the device - its key column (dim_table_rows rows, the keys of
     dim_keys) and its one GROUP BY column (whole numbers spanning at most 65536 values, the values of
     dim_group_values). With them, a dense join's dim-row pass runs on the device instead of the host. */
  const CqlColumn* dim_key_column;
  const CqlColumn* dim_group_column;
} CqlJoinAgg;

/* Groups come out in the order their first dim row is met; out_group_dim_row[g] is that row,
   out_results[g*expr_count + e] the aggregate. out_strategy receives 1 (dense), 2 (probe) or 3 (lookup table). */
int cqlops_join_aggregate(const CqlJoinAgg* query, uint64_t max_groups, uint64_t* out_groups, uint64_t* out_group_dim_row, double* out_results,
                          uint32_t* out_strategy);

/* The zone map of a numeric column (cql_column_ensure_zone_map; the CQL_ZoneMapChunk ranges scans
   prune with, src/query_exec/query_exec.c:13294-13540): for each chunk of CQLOPS_ZONEMAP_CHUNK_ROWS
   rows its smallest and largest value as f64 (min > max: a chunk with no values, all NaN) into
   out_zone_map[2 * chunk], then the largest min and the smallest max over the chunks with values;
   out_chunks >= ceil(rows / chunk rows) + 1 entries. Computed on the GPU. */
int cqlops_zone_map_build(const CqlColumn* column, double* out_zone_map, uint64_t out_chunks);

/* The zone-map pruning of an AND of leaves over a table held in one buffer
   (qe_scan_build_dispatch_ranges, query_exec.c:13307-13540): a chunk is skipped when a leaf proves it
   empty (qe_zonemap_chunk_is_prunable, :13294-13304); short interior gaps (< 1M rows) are scanned
   anyway; nothing is pruned unless 10% of the rows go; the kept chunks merge into ranges, or - when
   the ranges would cost more than one pass (4M rows each) - one range with a skip bitmap. Writes at
   most max_ranges ranges as (first row, end row) pairs; out_skip_bits (optional, one bit per chunk,
   ceil(chunks / 32) words) is filled and *out_use_skip set when the bitmap form is chosen. Returns the
   number of ranges (0 for an empty table). */
uint64_t cqlops_scan_ranges(const CqlColumn* columns, uint32_t column_count, const CqlLeaf* leaves, uint32_t leaf_count,
                            uint64_t* out_ranges, uint64_t max_ranges, uint32_t* out_skip_bits, int* out_use_skip,
                            uint64_t* out_pruned_rows);

/* qe_values_fixed_point (src/query_exec/query_exec.c:3893-3983) over a device column (or the rows of
   a selection): the smallest scale s <= 6 at which every value v is whole, that is (S64)(v*10^s +- 0.5)
   / 10^s == v, with every |v| < 2^31 and the largest |v| * 10^s < 2^31; -1 when there is none.
   U32/I32 columns have scale 0 while their magnitudes stay below 2^31. Returns 1 when it ran. */
int cqlops_fixed_scale(const CqlColumn* column, CqlBuffer* selection, uint64_t selection_count, int32_t* out_scale, double* out_largest);

/* GROUP BY one small-range whole-number key (U32/I32, or F64 holding whole numbers) with
   COUNT/SUM/AVG/MIN/MAX over F64/F32 arguments that are decimals of at most 6 places - the dense
   branch of qe_aggregate_impl with fixed-point arguments (query_exec.c:10896-11083, kernels
   aggregate_dense_f64/_f32). Each argument is scaled by 10^s and summed exactly as an integer; the
   values are finalized as there: SUM = (F64)sum / 10^s, AVG = (F64)sum / 10^s / count, MIN/MAX =
   (F64)(S32)q / 10^s, COUNT = count. Optional selection: selection_count u32 row numbers in a device
   buffer. Writes the present groups in key order: out_keys, out_first_rows (the smallest row of the
   group), out_counts and out_results[g * expr_count + e], at most max_groups of them; out_scales[e]
   (optional) receives each argument's scale. Refuses (returns 0 with cqlops_last_error set) when an
   argument is not fixed-point or the key range is too wide, as the reference then takes another path. */
int cqlops_group_dense_fixed(const CqlColumn* key, uint32_t expr_count, const uint32_t* funcs, const CqlColumn* const* args,
                             CqlBuffer* selection, uint64_t selection_count, uint64_t max_groups, uint64_t* out_groups,
                             int64_t* out_keys, uint64_t* out_first_rows, uint64_t* out_counts, double* out_results, int32_t* out_scales);

/* ORDER BY up to 4 numeric keys (desc[k] != 0 for DESC), keys compared as F64 values with ties broken
   by input position - qe_sort_rows (src/query_exec/query_exec.c:5376-6155, compare :4859-4882) with a
   stable LSD radix sort in place of the bitonic sorts. Without a selection the input is the columns' rows
   and the output their row numbers; with one (selection_count u32 row numbers in a device buffer, the
   row set of a filter) the input is those rows in selection order and the output is their row numbers.
   Writes up to out_capacity row numbers in sorted order. */
int cqlops_sort_rows(const CqlColumn* keys, uint32_t key_count, const uint32_t* desc, CqlBuffer* selection,
                     uint64_t selection_count, uint32_t* out_rows, uint64_t out_capacity);

/* Row materialization (selection_gather.comp modes 0/1, qe_selection_gather_column,
   src/query_exec/query_exec.c:4371-4410): the values of `count` selected rows of each column, in
   selection order, written to host memory. The selection is `rows` (host memory, e.g. a scan's out_rows),
   else the device buffer `selection` (count u32 row numbers), else rows 0..count-1. out_values[c] receives
   count values of column c: 4 bytes each for U32/I32/F32/DATE/ENUM columns, for narrow and sequence
   encodings (the value base + code or base + row) and for dictionary strings (the code); 8 bytes for
   U64/I64/F64/TIMESTAMP/DECIMAL; 1 byte for BOOL. Raw strings go through cqlops_gather_strings. Host rows
   are checked against the columns' length; a device selection's rows past a column read as zero. Outputs
   laid out as one block - column c at the byte offset that sums, over the columns before it, count x width
   rounded up to a multiple of 16 - come back in one read. */
int cqlops_gather_rows(const CqlColumn* columns, uint32_t column_count, const uint32_t* rows, CqlBuffer* selection, uint64_t count,
                       void* const* out_values);

/* The selected rows of a raw STRING8 column (bytes and u64 offsets), selection as cqlops_gather_rows:
   row i's bytes are out_bytes[out_offsets[i] .. out_offsets[i + 1]), out_offsets holding count + 1 values.
   *out_bytes_needed receives the selected bytes; when they exceed bytes_capacity nothing is written past
   the offsets' first entry and 0 is returned (call again with room). At most 4 GB of selected bytes. */
int cqlops_gather_strings(const CqlColumn* column, const uint32_t* rows, CqlBuffer* selection, uint64_t count, uint64_t* out_offsets,
                          char* out_bytes, uint64_t bytes_capacity, uint64_t* out_bytes_needed);

/* A HAVING condition over the grouped result, evaluated for every group at once (qk_having_kernel,
   src/query_exec/query_kernel.c:2530-2575): `condition` is an expression over v0..v7 (group i's values of
   the result columns, as doubles) and lit[0..15] (the literals), in C syntax (&&, ||, !, comparisons,
   arithmetic, fabs/fmin/fmax/floor/ceil/sqrt/isnan); out_keep[i] = 1 when group i passes. Conditions that
   differ only in their literals share one compiled kernel. Refuses a condition with anything else. */
/* The CUDA C++ source of the HAVING kernel for a condition over v0..v(column_count-1) and lit[]
   (qk_having_kernel, query_kernel.c:2530-2575): binding 0 keep (u32 per group), 1 the literals (f64),
   2 + c result column c (f64), push slot 0 the group count. Returns 0 when the condition uses anything
   but v0..v7, lit[i], numbers, operators and fabs/fmin/fmax/floor/ceil/sqrt/isnan, or cap is short. */
int cqlops_having_source(const char* condition, uint32_t column_count, char* out, uint64_t cap, uint64_t* out_len);
int cqlops_having(const char* condition, const double* literals, uint32_t literal_count, const double* const* columns, uint32_t column_count,
                  uint64_t group_count, uint32_t* out_keep);

/* ROW_NUMBER, RANK and DENSE_RANK over (PARTITION BY the first partition_key_count keys ORDER BY the
   rest) - qe_window_rank_gpu, src/query_exec/query_exec.c:6155-6540. The rows (or the selection's, as for
   cqlops_sort_rows) are ordered by all the keys as cqlops_sort_rows orders them; a position starts a
   partition when a partition key differs from the previous position's and a peer group when any key
   differs (keys compared as F64 with !=, window_rank_flags.comp). Per sorted position: out_rows the row
   number, out_row_number the position within its partition (from 1), out_rank 1 + the position of its
   peer group's first row within the partition, out_dense_rank the count of peer groups up to it in the
   partition. Every output (any may be NULL) must hold all the rows. */
int cqlops_window_rank(const CqlColumn* keys, uint32_t key_count, const uint32_t* desc, uint32_t partition_key_count, CqlBuffer* selection,
                       uint64_t selection_count, uint32_t* out_rows, uint32_t* out_row_number, uint32_t* out_rank, uint32_t* out_dense_rank,
                       uint64_t out_capacity);

/* Q filter/aggregate queries over one table in one shared scan: SELECT COUNT(*), SUM(col) WHERE
   <programs[q]> for q = 0 .. query_count-1 - the batched form of cqlops_fused_filter_aggregate
   (qe_fused_filter_aggregate, query_exec.c:9888-10254). Every program is built over `columns` (numeric,
   full width, one length; at most 10); sum_columns[q] is the summed column's index or -1 (COUNT only);
   a summed column needs its range (has_range). Queries are grouped by shape (the same bytecode up to
   literal values), one generated kernel evaluates each shape for its queries, literals become per-query
   thresholds. Counts are exact; sums are exact 128-bit sums of the values scaled by 2^k (k from the
   column's range, |value| x 2^k < 2^55), so |error| <= matched rows x 2^-(k+1); the scale does not
   depend on the form, so every form gives the same sums. rows_per_thread picks the form of the generated
   kernel: 4, 8 or 16 rows a thread in registers (plus 1 << 9 for 512-thread CTAs instead of 256), 0 the
   shared-memory tile form, or CQLOPS_BATCH_AUTOTUNE: the form timed fastest for the batch's plan shape,
   each candidate timed on the shape's first batches. out_shapes (optional) receives the shape count.
   Refuses programs with string comparisons. */
int cqlops_batch_filter_aggregate(const CqlProgram* const* programs, uint32_t query_count, const CqlColumn* columns, uint32_t column_count,
                                  const int32_t* sum_columns, uint32_t rows_per_thread, uint64_t* out_counts, double* out_sums,
                                  uint32_t* out_shapes);
#define CQLOPS_BATCH_AUTOTUNE 0xffffffffu
/* The form the calling thread's last batched scan ran in: rows a thread in bits 0-7 (0 the tile form),
   the block size / 256 in bits 8-15 (0 or 1: 256 threads), bit 16 set when the run was an autotuner trial. */
uint32_t cqlops_batch_last_form(void);
/* Forgets every tuned plan shape (each is timed again from its next batch). */
void cqlops_batch_tuner_reset(void);

/* A shape catalog for a stream of batches over one table: the WHERE shapes, column types and summed
   columns its batches have met, in the order met (at most 64 shapes). A batch run with a catalog
   compiles one kernel for all of the catalog's shapes - a shape absent from the batch has no queries -
   so batches of varying mixes of known shapes reuse one kernel; columns no query of a launch reads are
   not loaded. A batch the catalog cannot take (full, or a column read as another type) runs as without
   it. Safe to share between threads. */
typedef struct CqlBatchCatalog CqlBatchCatalog;
CqlBatchCatalog* cqlops_batch_catalog_create(void);
void cqlops_batch_catalog_destroy(CqlBatchCatalog* catalog);
uint32_t cqlops_batch_catalog_shapes(CqlBatchCatalog* catalog);

/* cqlops_batch_filter_aggregate through a catalog; the results are the same. */
int cqlops_batch_filter_aggregate_cat(CqlBatchCatalog* catalog, const CqlProgram* const* programs, uint32_t query_count,
                                      const CqlColumn* columns, uint32_t column_count, const int32_t* sum_columns, uint32_t rows_per_thread,
                                      uint64_t* out_counts, double* out_sums, uint32_t* out_shapes);

/* Enters the queries' shapes in the catalog and compiles its kernel, without running it (a prepared
   statement's compile step). */
int cqlops_batch_prepare(CqlBatchCatalog* catalog, const CqlProgram* const* programs, uint32_t query_count, const CqlColumn* columns,
                         uint32_t column_count, const int32_t* sum_columns, uint32_t rows_per_thread);

/* The sources of the cube kernels cqlops_batch_filter_aggregate would compile for these queries (no
   device work): which = 0 the answers, 1 + p table pass p (the cubes whose shared tables fit together
   are built by one pass; 0 is returned past the last). Queries whose WHERE reads only whole-number
   columns of small range (at most 4 columns, 65536 value combinations) are answered from a dense table of
   the rows - per combination, the row count and the 128-bit fixed-point sums - built in one pass; each
   such query tests its predicate on the combinations instead of the rows. out_cube_queries receives how
   many queries the cube answers. Returns 0 when none can be. */
int cqlops_batch_cube_source(const CqlProgram* const* programs, uint32_t query_count, const CqlColumn* columns, uint32_t column_count,
                             const int32_t* sum_columns, uint32_t which, char* out, uint64_t cap, uint64_t* out_len, uint32_t* out_cube_queries);

/* The CUDA C++ source cqlops_batch_filter_aggregate would compile for its first launch (no device
   work), up to cap bytes into out (out_len receives the length). rows_per_thread | CQLOPS_BATCH_PERSISTENT_SOURCE
   (a register form): the source of the persistent form (cqlops_batch_persist_create) instead. */
#define CQLOPS_BATCH_PERSISTENT_SOURCE 0x10000u
int cqlops_batch_source(const CqlProgram* const* programs, uint32_t query_count, const CqlColumn* columns, uint32_t column_count,
                        const int32_t* sum_columns, uint32_t rows_per_thread, char* out, uint64_t cap, uint64_t* out_len, uint32_t* out_shapes);

/* The persistent shared scan: the batched scan for a serving loop over one table, as one long-lived kernel
   instead of a launch per batch. The kernel (the register form, compiled for every shape of `catalog`)
   waits on the device for the next batch in a ring of parameter slots in device memory, scans the table
   for it, adds each CTA's exact integer totals into the slot's accumulators, and the CTA that finishes last
   writes the answers into page-locked host memory and marks the batch done; the host writes a batch's
   thresholds and literals with copies and polls its done word. The kernel returns by itself after idle_us
   microseconds without a batch (0: 2000) and is launched again by the next run; a batch that brings a shape
   new to the catalog recompiles it. Each wait is bounded: the device's by the idle limit, the host's by 5 s
   (then the run fails with an error). rows_per_thread: 4, 8 or 16 (the register form's rows per thread,
   256 threads a CTA). A run takes at most 384 queries of numeric WHERE shapes (no cube answers); its
   results equal cqlops_batch_filter_aggregate's bit for bit. Runs on one object are serialised. */
typedef struct CqlBatchPersist CqlBatchPersist;
CqlBatchPersist* cqlops_batch_persist_create(CqlBatchCatalog* catalog, const CqlColumn* columns, uint32_t column_count,
                                             uint32_t rows_per_thread, uint32_t idle_us);
int cqlops_batch_persist_run(CqlBatchPersist* p, const CqlProgram* const* programs, uint32_t query_count, const int32_t* sum_columns,
                             uint64_t* out_counts, double* out_sums);
/* batches run, kernel launches (the first and each after an idle return) and compiles so far */
void cqlops_batch_persist_stats(CqlBatchPersist* p, uint64_t* out_batches, uint64_t* out_launches, uint64_t* out_compiles);
/* the CTAs of the kernel's last launch (0 before the first) */
uint32_t cqlops_batch_persist_ctas(CqlBatchPersist* p);
/* ends the kernel (a stop word in the slot it waits on) and frees everything; 0 if it did not return in 5 s */
int cqlops_batch_persist_destroy(CqlBatchPersist* p);

/* ---- the resident chunk cache (QE_ResidentCache, src/query_exec/query_exec.c:1679-1970) ----
   Device copies of host column chunks kept between queries, found by (column, write generation, first
   row, rows, stored width). A miss makes room within the budget (the entries used only once first, the
   most recent of them first, then the least recently used; pinned entries are never taken) and copies
   the rows in; a chunk of a column written since (another generation) is never handed out and is freed
   when met. The budget is budget_bytes (0: 70 % of the device's memory), never more than the memory the
   allocator reports reachable less 512 MB. With ops NULL the buffers are cqlcuda buffers (acquire returns
   a CqlBuffer*) and the backend's eviction hook frees entries when another allocation does not fit;
   other ops put the same policy over any allocator. Safe to share between threads. */
typedef struct CqlResidentOps
{
  void* (*alloc)(void* ctx, uint64_t bytes);
  int (*copy)(void* ctx, void* buffer, const void* host, uint64_t bytes);   /* 1 on success */
  void (*release)(void* ctx, void* buffer);
  uint64_t (*total_memory)(void* ctx);   /* may be NULL */
  uint64_t (*free_memory)(void* ctx);    /* may be NULL */
  void* ctx;
} CqlResidentOps;

typedef struct CqlResidentStats
{
  uint64_t hit_bytes, miss_bytes, evicted_bytes, bytes_in_use, entries, budget_bytes;
} CqlResidentStats;

typedef struct CqlResident CqlResident;
CqlResident* cqlops_resident_create(uint64_t budget_bytes, const CqlResidentOps* ops);
void cqlops_resident_destroy(CqlResident* cache);
/* The chunk's buffer, pinned until cqlops_resident_release; *out_hit says whether it was cached. NULL
   when it cannot be held (the caller then streams the rows through a buffer of its own). */
void* cqlops_resident_acquire(CqlResident* cache, uint64_t column_uid, uint64_t generation, const void* host_rows, uint64_t row_start,
                              uint64_t rows, uint32_t width, int* out_hit);
void cqlops_resident_release(CqlResident* cache, const void* buffer);
/* Frees unpinned entries until bytes_wanted are freed or none is left; returns the bytes freed. */
uint64_t cqlops_resident_evict(CqlResident* cache, uint64_t bytes_wanted);
void cqlops_resident_clear(CqlResident* cache);
CqlResidentStats cqlops_resident_stats(CqlResident* cache);

/* A host column for the streamed operators: its identity in the cache (uid and write generation), its
   values, and - for a key or a summed column - the whole column's range. */
typedef struct CqlHostColumn
{
  uint64_t uid;
  uint64_t generation;
  const void* values;   /* `rows` values of `type` (U32, I32, F32 or F64) */
  uint32_t type;
  uint32_t has_range;
  double zone_min;
  double zone_max;
} CqlHostColumn;

/* cqlops_scan_simple over host columns streamed through the cache in chunks of chunk_rows (0: 16M):
   qe_scan_filter_streamed (src/query_exec/query_exec.c:2242-2494). Each chunk's columns come from the
   cache or are uploaded into it, the chunk is scanned, its rows are offset by the chunk's first row and
   appended in order; the count is the chunks' total. The same count and rows as the resident scan. */
int cqlops_scan_simple_streamed(CqlResident* cache, const CqlHostColumn* columns, uint32_t column_count, uint64_t rows, const CqlLeaf* leaves,
                                uint32_t leaf_count, uint64_t chunk_rows, uint64_t* out_count, uint32_t* out_rows, uint64_t out_capacity,
                                uint64_t* out_uploaded_bytes);

/* cqlops_group_dense over host columns streamed through the cache: qe_aggregate_dense_streamed
   (src/query_exec/query_exec.c:7984-8068). The groups are the key column's whole range (its zone), so
   every chunk's groups line up; counts and sums are added and minimums and maximums kept chunk by
   chunk, all in integers: the same results as the resident dense group-by. args[e] is NULL for COUNT;
   at most 8 aggregates over at most 4 distinct argument columns, as cqlops_group_dense. */
int cqlops_group_dense_streamed(CqlResident* cache, const CqlHostColumn* key, uint64_t rows, uint32_t expr_count, const uint32_t* funcs,
                                const CqlHostColumn* const* args, uint64_t chunk_rows, uint64_t max_groups, uint64_t* out_group_count,
                                int64_t* out_min_key, uint64_t* out_counts, int64_t* out_sums, int64_t* out_mins, int64_t* out_maxs,
                                uint64_t* out_uploaded_bytes);

/* cqlops_join_aggregate with the fact side (the key and the argument columns) streamed from the host
   through the cache: qe_join_probe_stream_core (src/query_exec/query_exec.c:8080-8420). Each chunk's
   fact-side totals - per key value over the key's whole range (dense, a range of at most 65536 values)
   or per dim row (the probe) - are added into running totals; the dim-row pass runs once at the end.
   query->fact_key and query->fact_args are not read; fact_args[e] is NULL where query->funcs[e] takes no
   fact column. The lookup-table strategy does not stream: strategy 3 is refused, 0 picks dense or probe. */
int cqlops_join_aggregate_streamed(CqlResident* cache, const CqlJoinAgg* query, const CqlHostColumn* fact_key,
                                   const CqlHostColumn* const* fact_args, uint64_t rows, uint64_t chunk_rows, uint64_t max_groups,
                                   uint64_t* out_groups, uint64_t* out_group_dim_row, double* out_results, uint32_t* out_strategy,
                                   uint64_t* out_uploaded_bytes);

/* SUM/MIN/MAX of a host column (U32/I32/F32/F64, rows values at host_values) streamed through the
   cache in chunks of chunk_rows (0: 16M) - qe_aggregate_global_streamed, src/query_exec/query_exec.c:
   8842-9112: each chunk's device copy comes from the cache (keyed by column_uid, generation and the
   chunk's rows) or is uploaded into it, and every workgroup partial of every chunk is added, in chunk
   then workgroup order, into one running sum, minimum and maximum that start at 0, +F64_MAX and
   -F64_MAX (qe_agg_stream_retire, :8812-8841; an empty column gives those sentinels). The cache must
   hold backend buffers (created with ops NULL). *out_uploaded_bytes (optional) receives the bytes copied
   to the device: 0 when every chunk was cached. */
int cqlops_aggregate_global_streamed(CqlResident* cache, uint64_t column_uid, uint64_t generation, const void* host_values, uint32_t type,
                                     uint64_t rows, uint64_t chunk_rows, double* out_sum, double* out_min, double* out_max,
                                     uint64_t* out_uploaded_bytes);

/* Why the last operator call returned 0 when it refused the request itself ("" otherwise; GPU
   failures are in cqlcuda_last_error()). */
const char* cqlops_last_error(void);

/* Count of kernel launches of the last operator call (for the bench's gpu_launches figure). */
uint32_t cqlops_last_launches(void);

#ifdef __cplusplus
}
#endif

#endif /* CQLOPS_H */
