/*
 * cql_ops_internal.h - declarations the operator layer's translation units share (not part of the C ABI).
 */
#ifndef CQL_OPS_INTERNAL_H
#define CQL_OPS_INTERNAL_H

#include "cqlops.h"

/* records why the current operator call refused the request (cqlops_last_error) */
void cqlops_note_error(const char* why);

/* 1 when a row count fits the kernels' 32-bit row numbers; else 0 with the reason noted */
int cqlops_rows_fit(uint64_t rows);

/* enqueues into batch b the rows of a selection bitmap of `rows` bits (bit i = row first_row + i), ascending,
   into `list` (at most its size / 4 of them) - cql_ops.c */
int cqlops_bitmap_rows_enqueue(CqlBatch* b, CqlBuffer* bitmap, uint64_t first_row, uint64_t rows, CqlBuffer* list);

/* result pairs put in order on the device by the radix sort (cql_ops_sort.c) */
int cqlops_sort_pairs(CqlBuffer* records, uint64_t n, uint32_t stride_words, uint32_t first_word, uint32_t second_word, int by_second,
                      uint32_t* out, uint64_t out_capacity);

/* The dense group-by's totals left on the device for a caller's next operations: the counts (u64 per group,
   from 0), the sums (two u32 words per group and expression) at sum_at, MIN and MAX (i32 per group and
   expression) at min_at / max_at. keep_open: the batch is left open for the caller, who ends it. */
typedef struct
{
  CqlBuffer* buffer;
  uint64_t sum_at, min_at, max_at;
  uint64_t group_count;
  int64_t min_key;
  int keep_open;      /* in: leave the batch open for the caller's next operations */
  CqlBatch* batch;    /* out (keep_open): that batch, which the caller ends */
} CqlDenseTotals;

int cql_group_dense_device(const CqlColumn* key, uint64_t rows, uint32_t expr_count, const uint32_t* funcs, const CqlColumn* const* arg_cols,
                           uint64_t max_groups, CqlDenseTotals* out);

#endif
