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

/* A device-resident column. `width` is the encoding the kernels are told
   (qe_encoding_shader_width, query_exec.c:1593-1601): 0 = stored as is, 1/2 = narrow codes of that
   many bytes with value = base + code, 3 = a sequence (value = base + row number, nothing stored).
   zone_min/zone_max stand in for the zone map range (qe_column_range_from_zone_map). */
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
} CqlColumn;

/* One comparison `column op target` of an AND-only filter (the leaves qe_scan_filter_selected
   hands to scan_simple, query_exec.c:2566-2680). */
typedef struct CqlLeaf
{
  uint32_t column;    /* index into the column array */
  uint32_t op;        /* CQLOPS_CMP_* */
  double target;
} CqlLeaf;

/* SUM/MIN/MAX of up to 4 whole columns (qe_aggregate_global_streamed, query_exec.c:8842-9112, one
   chunk). Partials are folded in workgroup order. Sequence columns are summed in closed form. */
int cqlops_aggregate_global(const CqlColumn* columns, uint32_t column_count, double* out_sum, double* out_min, double* out_max);

/* AND of up to 8 numeric comparisons over up to 10 columns with scan_simple
   (qe_scan_filter_selected, query_exec.c:2495-3276). Writes the match count; when out_rows is not
   NULL and out_capacity > 0 also up to out_capacity matching row numbers in ascending order (the
   kernel's order is not deterministic; the list is sorted before it is returned).
   When out_rows is NULL the kernel runs count-only. */
int cqlops_scan_simple(const CqlColumn* columns, uint32_t column_count, const CqlLeaf* leaves, uint32_t leaf_count,
                       uint64_t* out_count, uint32_t* out_rows, uint64_t out_capacity);

/* GROUP BY one small-range whole-number key with COUNT/SUM/AVG/MIN/MAX over whole-number
   columns (qe_dense_stream_core, query_exec.c:7632-7983, one chunk). funcs[e]/arg_cols[e] describe
   expression e (arg_cols[e] is ignored for COUNT). Outputs, per group g = key - min_key:
   out_counts[g], out_sums[g*exprs+e] (64-bit two's complement), out_mins/out_maxs[g*exprs+e]
   (INT32_MAX / INT32_MIN when the group has no rows). out_group_count receives the group count;
   the output arrays must hold max_groups entries (times exprs). */
int cqlops_group_dense(const CqlColumn* key, uint64_t rows, uint32_t expr_count, const uint32_t* funcs, const CqlColumn* const* arg_cols,
                       uint64_t max_groups, uint64_t* out_group_count, int64_t* out_min_key, uint64_t* out_counts, int64_t* out_sums,
                       int64_t* out_mins, int64_t* out_maxs);

/* Count of kernel launches of the last operator call (for the bench's gpu_launches figure). */
uint32_t cqlops_last_launches(void);

#ifdef __cplusplus
}
#endif

#endif /* CQLOPS_H */
