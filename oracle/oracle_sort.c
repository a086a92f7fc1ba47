/*
 * oracle_sort.c - ORDER BY as the reference orders rows (TEST INFRASTRUCTURE ONLY).
 *
 * Every numeric key is compared as an F64 with < and > (qe_sort_rows_compare_ctx,
 * src/query_exec/query_exec.c:4859-4882), a DESC key negates the comparison, and rows that compare
 * equal on every key keep their input order (qe_order_before, query_exec.c:4890-4903). The rows are
 * put in that order by a bottom-up merge sort (qe_order_merge_sort, query_exec.c:4905-4940).
 */
#include "oracle.h"

#include <stdlib.h>

static int orc_sort_compare(const double* keys, uint32_t key_count, const uint32_t* desc, uint64_t rows, uint64_t a, uint64_t b)
{
  for (uint32_t k = 0; k < key_count; k++)
  {
    double va = keys[(uint64_t)k * rows + a], vb = keys[(uint64_t)k * rows + b];
    int cmp = va < vb ? -1 : va > vb ? 1 : 0;
    if (cmp) return desc && desc[k] ? -cmp : cmp;
  }
  return a < b ? -1 : a > b ? 1 : 0;
}

int orc_sort_rows(const double* keys, uint32_t key_count, const uint32_t* desc, uint64_t rows, uint64_t* out)
{
  uint64_t* buf = (uint64_t*)malloc((rows ? rows : 1) * sizeof(uint64_t));
  if (!buf) return 0;
  for (uint64_t i = 0; i < rows; i++) out[i] = i;
  uint64_t* src = out;
  uint64_t* dst = buf;
  for (uint64_t width = 1; width < rows; width *= 2)
  {
    for (uint64_t start = 0; start < rows; start += 2 * width)
    {
      uint64_t mid = start + width < rows ? start + width : rows;
      uint64_t end = start + 2 * width < rows ? start + 2 * width : rows;
      uint64_t l = start, r = mid, o = start;
      while (l < mid && r < end)
        dst[o++] = orc_sort_compare(keys, key_count, desc, rows, src[r], src[l]) < 0 ? src[r++] : src[l++];
      while (l < mid) dst[o++] = src[l++];
      while (r < end) dst[o++] = src[r++];
    }
    uint64_t* t = src;
    src = dst;
    dst = t;
  }
  if (src != out)
    for (uint64_t i = 0; i < rows; i++) out[i] = src[i];
  free(buf);
  return 1;
}

/* ROW_NUMBER / RANK / DENSE_RANK as the reference computes them (qe_window_rank_gpu,
   src/query_exec/query_exec.c:6155-6216 and window_rank_flags.comp): the rows in the ORDER BY order
   above, a position starting a partition when a partition key differs from the previous row's and a peer
   group when any key differs (F64 !=), then one pass: row number from the partition start, rank from the
   peer group's start, dense rank counting peer groups. */
int orc_window_rank(const double* keys, uint32_t key_count, const uint32_t* desc, uint32_t partition_count, uint64_t rows, uint64_t* out_rows,
                    uint32_t* row_number, uint32_t* rank, uint32_t* dense_rank)
{
  if (!orc_sort_rows(keys, key_count, desc, rows, out_rows)) return 0;
  uint64_t part_start = 0, peer_start = 0;
  uint32_t dense = 0;
  for (uint64_t i = 0; i < rows; i++)
  {
    int new_part = i == 0, new_peer = i == 0;
    for (uint32_t k = 0; i > 0 && k < key_count; k++)
    {
      double a = keys[(uint64_t)k * rows + out_rows[i - 1]], b = keys[(uint64_t)k * rows + out_rows[i]];
      if (a != b)
      {
        new_peer = 1;
        if (k < partition_count) new_part = 1;
      }
    }
    if (new_part)
    {
      part_start = i;
      peer_start = i;
      dense = 1;
    }
    else if (new_peer)
    {
      peer_start = i;
      dense += 1;
    }
    row_number[i] = (uint32_t)(i - part_start + 1);
    rank[i] = (uint32_t)(peer_start - part_start + 1);
    dense_rank[i] = dense;
  }
  return 1;
}
