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
