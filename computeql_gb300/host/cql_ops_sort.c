/*
 * cql_ops_sort.c - ORDER BY up to 4 numeric keys, ties by input position (qe_sort_rows,
 * src/query_exec/query_exec.c:5376-6155; the tie rule of the generated sort, query_kernel.c:2156-2177),
 * as a stable LSD radix sort on the GPU: the last key first, each key 8 bits per pass.
 */
#include "cqlops.h"

#include <stdio.h>
#include <stdlib.h>
#include <string.h>

#define SORT_TILE 4096
#define QE_GPU_WORKGROUP_SIZE 256

void cqlops_note_error(const char* why);

static int refuse(const char* why)
{
  cqlops_note_error(why);
  return 0;
}

static CqlBuffer* pooled(const char* name, uint64_t size, uint32_t flags)
{
  return cqlcuda_buffer_alloc_pooled(name, (uint64_t)strlen(name), size ? size : 8, flags, NULL);
}

static int key_bytes(uint32_t type)
{
  switch (type)
  {
    case CQLOPS_TYPE_U32: case CQLOPS_TYPE_I32: case CQLOPS_TYPE_F32: case 9: case 12: return 4;
    case CQLOPS_TYPE_U64: case CQLOPS_TYPE_I64: case CQLOPS_TYPE_F64: case 10: case 11: return 8;
    default: return 0;
  }
}

int cqlops_sort_rows(const CqlColumn* keys, uint32_t key_count, const uint32_t* desc, CqlBuffer* selection,
                     uint64_t selection_count, uint32_t* out_rows, uint64_t out_capacity)
{
  cqlops_note_error("");
  if (key_count == 0 || key_count > 4) return refuse("1 to 4 sort keys");
  uint64_t rows = keys[0].rows;
  uint64_t n = selection ? selection_count : rows;
  if (rows >= 0xffffffffull || n >= 0xffffffffull) return refuse("row count out of range");
  uint32_t widest = 4;
  for (uint32_t k = 0; k < key_count; k++)
  {
    int narrow_ok = keys[k].width == 0 || (keys[k].width <= 3 && key_bytes(keys[k].type) == 4 && keys[k].type != CQLOPS_TYPE_F32);
    if (keys[k].rows != rows || (!keys[k].buffer && keys[k].width != 3) || !narrow_ok || !key_bytes(keys[k].type))
      return refuse("sort keys are numeric columns of the same length (narrow encodings only for 32-bit integers)");
    if (key_bytes(keys[k].type) > (int)widest) widest = 8;
  }
  if (selection && cqlcuda_buffer_size(selection) < n * 4) return refuse("selection buffer smaller than its count");
  if (n == 0) return 1;
  uint64_t tiles = (n + SORT_TILE - 1) / SORT_TILE;
  uint64_t hist_n = tiles * 256;
  CqlBuffer* perm[2] = { pooled("sort_perm_a", n * 4, CQLCUDA_BUFFER_READ_WRITE), pooled("sort_perm_b", n * 4, CQLCUDA_BUFFER_READ_WRITE) };
  CqlBuffer* kbuf[2] = { pooled("sort_keys_a", n * widest, CQLCUDA_BUFFER_READ_WRITE), pooled("sort_keys_b", n * widest, CQLCUDA_BUFFER_READ_WRITE) };
  CqlBuffer* hist = pooled("sort_hist", hist_n * 4, CQLCUDA_BUFFER_READ_WRITE);
  CqlBuffer* offsets = pooled("sort_offsets", (hist_n + 1) * 4, CQLCUDA_BUFFER_READ_WRITE);
  CqlBuffer* cursor = pooled("sort_cursor", hist_n * 4, CQLCUDA_BUFFER_READ_WRITE);
  CqlBuffer* block_sums = pooled("sort_block_sums", ((hist_n + 255) / 256) * 4, CQLCUDA_BUFFER_READ_WRITE);
  CqlKernel* kkeys = cqlcuda_kernel_alloc("cql_sort_keys", 13);
  CqlKernel* kcount = cqlcuda_kernel_alloc("cql_radix_count", 15);
  CqlKernel* kscan = cqlcuda_kernel_alloc("prefix_sum", 10);
  CqlKernel* kscatter = cqlcuda_kernel_alloc("cql_radix_scatter", 17);
  if (!perm[0] || !perm[1] || !kbuf[0] || !kbuf[1] || !hist || !offsets || !cursor || !block_sums || !kkeys || !kcount || !kscan || !kscatter)
    return 0;
  CqlBuffer* sel = selection ? selection : perm[0];
  int cur = 0;
  CqlBatch* b = cqlcuda_batch_begin(0, n * 4);
  for (int k = (int)key_count - 1; k >= 0; k--)
  {
    int kb = key_bytes(keys[k].type);
    /* the key in the current order (the first key sorted builds the identity permutation) */
    cqlcuda_kernel_set_arg_buffer(kkeys, 0, keys[k].buffer ? keys[k].buffer : perm[cur]);
    cqlcuda_kernel_set_arg_buffer(kkeys, 1, perm[cur]);
    cqlcuda_kernel_set_arg_buffer(kkeys, 2, kbuf[cur]);
    cqlcuda_kernel_set_arg_buffer(kkeys, 3, sel);
    cqlcuda_kernel_set_arg_u64(kkeys, 0, n);
    cqlcuda_kernel_set_arg_u64(kkeys, 1, keys[k].type);
    cqlcuda_kernel_set_arg_u64(kkeys, 2, desc && desc[k] ? 1 : 0);
    cqlcuda_kernel_set_arg_u64(kkeys, 3, k == (int)key_count - 1 ? 0 : 1);
    cqlcuda_kernel_set_arg_u64(kkeys, 4, selection ? 1 : 0);
    cqlcuda_kernel_set_arg_u64(kkeys, 5, keys[k].width);
    cqlcuda_kernel_set_arg_u64(kkeys, 6, keys[k].base);
    cqlcuda_batch_kernel_execute(b, kkeys, (uint32_t)n, QE_GPU_WORKGROUP_SIZE);
    for (int p = 0; p < kb; p++)
    {
      int last = k == 0 && p == kb - 1;
      cqlcuda_kernel_set_arg_buffer(kcount, 0, kbuf[cur]);
      cqlcuda_kernel_set_arg_buffer(kcount, 1, hist);
      cqlcuda_kernel_set_arg_u64(kcount, 0, n);
      cqlcuda_kernel_set_arg_u64(kcount, 1, (uint64_t)(8 * p));
      cqlcuda_kernel_set_arg_u64(kcount, 2, (uint64_t)kb);
      cqlcuda_batch_kernel_execute(b, kcount, (uint32_t)(tiles * 256), 256);
      cqlcuda_kernel_set_arg_buffer(kscan, 0, hist);
      cqlcuda_kernel_set_arg_buffer(kscan, 1, offsets);
      cqlcuda_kernel_set_arg_buffer(kscan, 2, cursor);
      cqlcuda_kernel_set_arg_buffer(kscan, 3, block_sums);
      cqlcuda_kernel_set_arg_u64(kscan, 0, hist_n);
      for (uint32_t mode = 0; mode < 3; mode++)
      {
        cqlcuda_kernel_set_arg_u64(kscan, 1, mode);
        cqlcuda_batch_kernel_execute(b, kscan, mode == 1 ? 256u : (uint32_t)(((hist_n + 255) / 256) * 256), 256);
      }
      cqlcuda_kernel_set_arg_buffer(kscatter, 0, kbuf[cur]);
      cqlcuda_kernel_set_arg_buffer(kscatter, 1, perm[cur]);
      cqlcuda_kernel_set_arg_buffer(kscatter, 2, kbuf[cur ^ 1]);
      cqlcuda_kernel_set_arg_buffer(kscatter, 3, perm[cur ^ 1]);
      cqlcuda_kernel_set_arg_buffer(kscatter, 4, offsets);
      cqlcuda_kernel_set_arg_buffer(kscatter, 5, sel);
      cqlcuda_kernel_set_arg_u64(kscatter, 0, n);
      cqlcuda_kernel_set_arg_u64(kscatter, 1, (uint64_t)(8 * p));
      cqlcuda_kernel_set_arg_u64(kscatter, 2, (uint64_t)kb);
      cqlcuda_kernel_set_arg_u64(kscatter, 3, last && selection ? 1 : 0);
      cqlcuda_kernel_set_arg_u64(kscatter, 4, last ? 1 : 0);
      cqlcuda_batch_kernel_execute(b, kscatter, (uint32_t)(tiles * 256), 256);
      cur ^= 1;
    }
  }
  uint64_t m = n < out_capacity ? n : out_capacity;
  if (out_rows && m) cqlcuda_batch_buffer_read(b, perm[cur], out_rows, m * 4);
  return cqlcuda_batch_end(b);
}
