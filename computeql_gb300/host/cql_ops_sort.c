/*
 * cql_ops_sort.c - ORDER BY up to 4 numeric keys, ties by input position (qe_sort_rows,
 * src/query_exec/query_exec.c:5376-6155; the tie rule of the generated sort, query_kernel.c:2156-2177),
 * as a stable LSD radix sort on the GPU: the last key first, each key 8 bits per pass.
 */
#include "cqlops.h"
#include "cql_ops_internal.h"

#include <stdio.h>
#include <stdlib.h>
#include <string.h>

#define SORT_TILE 4096
#define QE_GPU_WORKGROUP_SIZE 256

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

/* The sort's checks and scratch; 0 (with the reason noted) when the keys cannot be sorted. */
static int sort_check(const CqlColumn* keys, uint32_t key_count, CqlBuffer* selection, uint64_t selection_count, uint64_t* out_n)
{
  if (key_count == 0 || key_count > 4) return refuse("1 to 4 sort keys");
  uint64_t rows = keys[0].rows;
  uint64_t n = selection ? selection_count : rows;
  if (!cqlops_rows_fit(rows) || !cqlops_rows_fit(n)) return 0;
  for (uint32_t k = 0; k < key_count; k++)
  {
    int narrow_ok = keys[k].width == 0 || (keys[k].width <= 3 && key_bytes(keys[k].type) == 4 && keys[k].type != CQLOPS_TYPE_F32);
    if (keys[k].rows != rows || (!keys[k].buffer && keys[k].width != 3) || !narrow_ok || !key_bytes(keys[k].type))
      return refuse("sort keys are numeric columns of the same length (narrow encodings only for 32-bit integers)");
  }
  if (selection && cqlcuda_buffer_size(selection) < n * 4) return refuse("selection buffer smaller than its count");
  *out_n = n;
  return 1;
}

/* Queues the stable LSD radix sort of n > 0 rows into batch b; *out_sorted receives the buffer that holds
   the row numbers in sorted order when the batch has run. */
static int sort_enqueue(CqlBatch* b, const CqlColumn* keys, uint32_t key_count, const uint32_t* desc, CqlBuffer* selection, uint64_t n,
                        CqlBuffer** out_sorted)
{
  uint32_t widest = 4;
  for (uint32_t k = 0; k < key_count; k++)
    if (key_bytes(keys[k].type) > (int)widest) widest = 8;
  uint64_t tiles = (n + SORT_TILE - 1) / SORT_TILE;
  uint64_t hist_n = tiles * 256;
  CqlBuffer* perm[2] = { pooled("sort_perm_a", n * 4, CQLCUDA_BUFFER_READ_WRITE), pooled("sort_perm_b", n * 4, CQLCUDA_BUFFER_READ_WRITE) };
  CqlBuffer* kbuf[2] = { pooled("sort_keys_a", n * widest, CQLCUDA_BUFFER_READ_WRITE), pooled("sort_keys_b", n * widest, CQLCUDA_BUFFER_READ_WRITE) };
  CqlBuffer* hist = pooled("sort_hist", hist_n * 4, CQLCUDA_BUFFER_READ_WRITE);
  CqlBuffer* offsets = pooled("sort_offsets", hist_n * 4, CQLCUDA_BUFFER_READ_WRITE);
  CqlBuffer* totals = pooled("sort_digit_totals", 8 * 256 * 4, CQLCUDA_BUFFER_READ_WRITE);
  CqlKernel* kkeys = cqlcuda_kernel_alloc("cql_sort_keys", 13);
  CqlKernel* kcount = cqlcuda_kernel_alloc("cql_radix_count", 15);
  CqlKernel* koffsets = cqlcuda_kernel_alloc("cql_radix_offsets", 17);
  CqlKernel* kscatter = cqlcuda_kernel_alloc("cql_radix_scatter", 17);
  if (!perm[0] || !perm[1] || !kbuf[0] || !kbuf[1] || !hist || !offsets || !totals || !kkeys || !kcount || !koffsets || !kscatter)
    return 0;
  CqlBuffer* sel = selection ? selection : perm[0];
  int cur = 0;
  for (int k = (int)key_count - 1; k >= 0; k--)
  {
    int kb = key_bytes(keys[k].type);
    int first_key = k == (int)key_count - 1;
    /* each pass's digit totals start at zero: the key pass counts the first digit, the count kernels the rest */
    cqlcuda_batch_fill_range(b, totals, 0, (uint64_t)kb * 256 * 4, 0);
    /* the key in the current order, with its first digit counted (the first key sorted starts from the
       identity permutation, which the first scatter takes as row numbers) */
    cqlcuda_kernel_set_arg_buffer(kkeys, 0, keys[k].buffer ? keys[k].buffer : perm[cur]);
    cqlcuda_kernel_set_arg_buffer(kkeys, 1, perm[cur]);
    cqlcuda_kernel_set_arg_buffer(kkeys, 2, kbuf[cur]);
    cqlcuda_kernel_set_arg_buffer(kkeys, 3, sel);
    cqlcuda_kernel_set_arg_buffer(kkeys, 4, hist);
    cqlcuda_kernel_set_arg_buffer(kkeys, 5, totals);
    cqlcuda_kernel_set_arg_u64(kkeys, 0, n);
    cqlcuda_kernel_set_arg_u64(kkeys, 1, keys[k].type);
    cqlcuda_kernel_set_arg_u64(kkeys, 2, desc && desc[k] ? 1 : 0);
    cqlcuda_kernel_set_arg_u64(kkeys, 3, first_key ? 0 : 1);
    cqlcuda_kernel_set_arg_u64(kkeys, 4, selection ? 1 : 0);
    cqlcuda_kernel_set_arg_u64(kkeys, 5, keys[k].width);
    cqlcuda_kernel_set_arg_u64(kkeys, 6, keys[k].base);
    cqlcuda_kernel_set_arg_u64(kkeys, 7, first_key ? 3 : 1);
    cqlcuda_batch_kernel_execute(b, kkeys, (uint32_t)n, QE_GPU_WORKGROUP_SIZE);
    for (int p = 0; p < kb; p++)
    {
      int last = k == 0 && p == kb - 1;
      uint64_t pass_totals = (uint64_t)p * 256 * 4;
      if (p > 0)
      {
        cqlcuda_kernel_set_arg_buffer(kcount, 0, kbuf[cur]);
        cqlcuda_kernel_set_arg_buffer(kcount, 1, hist);
        cqlcuda_kernel_set_arg_buffer_range(kcount, 2, totals, pass_totals, 256 * 4);
        cqlcuda_kernel_set_arg_u64(kcount, 0, n);
        cqlcuda_kernel_set_arg_u64(kcount, 1, (uint64_t)(8 * p));
        cqlcuda_kernel_set_arg_u64(kcount, 2, (uint64_t)kb);
        cqlcuda_batch_kernel_execute(b, kcount, (uint32_t)(tiles * 256), 256);
      }
      cqlcuda_kernel_set_arg_buffer(koffsets, 0, hist);
      cqlcuda_kernel_set_arg_buffer_range(koffsets, 1, totals, pass_totals, 256 * 4);
      cqlcuda_kernel_set_arg_buffer(koffsets, 2, offsets);
      cqlcuda_kernel_set_arg_u64(koffsets, 0, n);
      cqlcuda_batch_kernel_execute(b, koffsets, 256u * 512u, 512);
      cqlcuda_kernel_set_arg_buffer(kscatter, 0, kbuf[cur]);
      cqlcuda_kernel_set_arg_buffer(kscatter, 1, perm[cur]);
      cqlcuda_kernel_set_arg_buffer(kscatter, 2, kbuf[cur ^ 1]);
      cqlcuda_kernel_set_arg_buffer(kscatter, 3, perm[cur ^ 1]);
      cqlcuda_kernel_set_arg_buffer(kscatter, 4, offsets);
      cqlcuda_kernel_set_arg_buffer(kscatter, 5, sel);
      cqlcuda_kernel_set_arg_buffer_range(kscatter, 6, totals, pass_totals, 256 * 4);
      cqlcuda_kernel_set_arg_u64(kscatter, 0, n);
      cqlcuda_kernel_set_arg_u64(kscatter, 1, (uint64_t)(8 * p));
      cqlcuda_kernel_set_arg_u64(kscatter, 2, (uint64_t)kb);
      cqlcuda_kernel_set_arg_u64(kscatter, 3, last && selection ? 1 : 0);
      cqlcuda_kernel_set_arg_u64(kscatter, 4, last ? 1 : 0);
      cqlcuda_kernel_set_arg_u64(kscatter, 5, first_key && p == 0 ? 1 : 0);
      cqlcuda_batch_kernel_execute(b, kscatter, (uint32_t)(tiles * 256), 256);
      cur ^= 1;
    }
  }
  *out_sorted = perm[cur];
  return 1;
}

int cqlops_sort_rows(const CqlColumn* keys, uint32_t key_count, const uint32_t* desc, CqlBuffer* selection,
                     uint64_t selection_count, uint32_t* out_rows, uint64_t out_capacity)
{
  cqlops_note_error("");
  uint64_t n = 0;
  if (!sort_check(keys, key_count, selection, selection_count, &n)) return 0;
  if (n == 0) return 1;
  CqlBatch* b = cqlcuda_batch_begin(0, n * 4);
  CqlBuffer* sorted = NULL;
  if (!sort_enqueue(b, keys, key_count, desc, selection, n, &sorted))
  {
    cqlcuda_batch_end(b);
    return 0;
  }
  uint64_t m = n < out_capacity ? n : out_capacity;
  if (out_rows && m) cqlcuda_batch_buffer_read(b, sorted, out_rows, m * 4);
  return cqlcuda_batch_end(b);
}

/* Result pairs put in order on the device (the join's pair output, the scan's rows with their scores): n
   records of stride_words u32 words in `records`; the pair (word first_word, word second_word) of each,
   sorted by the first word then the second (by_second) or by the first alone (ties by position) with the
   radix sort above, and up to out_capacity sorted pairs (first, second) read into out. */
int cqlops_sort_pairs(CqlBuffer* records, uint64_t n, uint32_t stride_words, uint32_t first_word, uint32_t second_word, int by_second,
                      uint32_t* out, uint64_t out_capacity)
{
  if (n == 0 || out_capacity == 0) return 1;
  if (!cqlops_rows_fit(n)) return 0;
  CqlBuffer* first = pooled("pairs_first", n * 4, CQLCUDA_BUFFER_READ_WRITE);
  CqlBuffer* second = pooled("pairs_second", n * 4, CQLCUDA_BUFFER_READ_WRITE);
  CqlBuffer* packed = pooled("pairs_sorted", n * 8, CQLCUDA_BUFFER_READ_WRITE);
  CqlKernel* unpack = cqlcuda_kernel_alloc("cql_pairs_unpack", 16);
  CqlKernel* pack = cqlcuda_kernel_alloc("cql_pairs_pack", 14);
  if (!first || !second || !packed || !unpack || !pack) return 0;
  CqlColumn keys[2];
  memset(keys, 0, sizeof(keys));
  for (int k = 0; k < 2; k++)
  {
    keys[k].type = CQLOPS_TYPE_U32;
    keys[k].rows = n;
    keys[k].buffer = k ? second : first;
  }
  uint64_t m = n < out_capacity ? n : out_capacity;
  CqlBatch* b = cqlcuda_batch_begin(0, m * 8);
  cqlcuda_kernel_set_arg_buffer(unpack, 0, records);
  cqlcuda_kernel_set_arg_buffer(unpack, 1, first);
  cqlcuda_kernel_set_arg_buffer(unpack, 2, second);
  cqlcuda_kernel_set_arg_u64(unpack, 0, n);
  cqlcuda_kernel_set_arg_u64(unpack, 1, stride_words);
  cqlcuda_kernel_set_arg_u64(unpack, 2, first_word);
  cqlcuda_kernel_set_arg_u64(unpack, 3, second_word);
  cqlcuda_batch_kernel_execute(b, unpack, (uint32_t)n, QE_GPU_WORKGROUP_SIZE);
  CqlBuffer* sorted = NULL;
  if (!sort_enqueue(b, keys, by_second ? 2u : 1u, NULL, NULL, n, &sorted))
  {
    cqlcuda_batch_end(b);
    return 0;
  }
  cqlcuda_kernel_set_arg_buffer(pack, 0, sorted);
  cqlcuda_kernel_set_arg_buffer(pack, 1, first);
  cqlcuda_kernel_set_arg_buffer(pack, 2, second);
  cqlcuda_kernel_set_arg_buffer(pack, 3, packed);
  cqlcuda_kernel_set_arg_u64(pack, 0, n);
  cqlcuda_batch_kernel_execute(b, pack, (uint32_t)n, QE_GPU_WORKGROUP_SIZE);
  cqlcuda_batch_buffer_read(b, packed, out, m * 8);
  return cqlcuda_batch_end(b);
}

/* ROW_NUMBER, RANK and DENSE_RANK (qe_window_rank_gpu, src/query_exec/query_exec.c:6155-6540): the rows
   sorted by (partition keys, order keys) with the sort above, then per sorted position whether it starts a
   partition or a peer group (keys compared as F64 with !=, window_rank_flags.comp), then the three ranks by
   one scan over the positions - all in one batch. */
#define WIN_TILE 2048u
#define WIN_AGG_BYTES 24u

int cqlops_window_rank(const CqlColumn* keys, uint32_t key_count, const uint32_t* desc, uint32_t partition_key_count, CqlBuffer* selection,
                       uint64_t selection_count, uint32_t* out_rows, uint32_t* out_row_number, uint32_t* out_rank, uint32_t* out_dense_rank,
                       uint64_t out_capacity)
{
  cqlops_note_error("");
  uint64_t n = 0;
  if (partition_key_count > key_count) return refuse("more partition keys than keys");
  if (!sort_check(keys, key_count, selection, selection_count, &n)) return 0;
  if (n == 0) return 1;
  if (out_capacity < n) return refuse("the outputs must hold every row");
  uint64_t tiles = (n + WIN_TILE - 1) / WIN_TILE;
  CqlBuffer* flags = pooled("window_flags", n, CQLCUDA_BUFFER_READ_WRITE);
  CqlBuffer* agg = pooled("window_tiles", tiles * WIN_AGG_BYTES, CQLCUDA_BUFFER_READ_WRITE);
  CqlBuffer* carry = pooled("window_carry", tiles * WIN_AGG_BYTES, CQLCUDA_BUFFER_READ_WRITE);
  CqlBuffer* ranks = pooled("window_ranks", n * 12, CQLCUDA_BUFFER_READ_WRITE);
  CqlKernel* kflags = cqlcuda_kernel_alloc("cql_window_flags", 16);
  CqlKernel* ktiles = cqlcuda_kernel_alloc("cql_window_tiles", 16);
  CqlKernel* kcarry = cqlcuda_kernel_alloc("cql_window_carry", 16);
  CqlKernel* kapply = cqlcuda_kernel_alloc("cql_window_apply", 16);
  if (!flags || !agg || !carry || !ranks || !kflags || !ktiles || !kcarry || !kapply) return 0;
  CqlBatch* b = cqlcuda_batch_begin(0, n * 16);
  CqlBuffer* sorted = NULL;
  if (!sort_enqueue(b, keys, key_count, desc, selection, n, &sorted))
  {
    cqlcuda_batch_end(b);
    return 0;
  }
  uint32_t types = 0, widths = 0;
  for (uint32_t k = 0; k < key_count; k++)
  {
    types |= (keys[k].type & 0xffu) << (8 * k);
    widths |= (keys[k].width & 0xffu) << (8 * k);
  }
  cqlcuda_kernel_set_arg_buffer(kflags, 0, sorted);
  cqlcuda_kernel_set_arg_buffer(kflags, 1, flags);
  for (uint32_t k = 0; k < 4; k++)
    cqlcuda_kernel_set_arg_buffer(kflags, 2 + k, k < key_count && keys[k].buffer ? keys[k].buffer : sorted);
  cqlcuda_kernel_set_arg_u64(kflags, 0, n);
  cqlcuda_kernel_set_arg_u64(kflags, 1, (uint64_t)key_count | (uint64_t)partition_key_count << 32);
  cqlcuda_kernel_set_arg_u64(kflags, 2, (uint64_t)types | (uint64_t)widths << 32);
  cqlcuda_kernel_set_arg_u64(kflags, 3, (uint64_t)(key_count > 0 ? keys[0].base : 0) | (uint64_t)(key_count > 1 ? keys[1].base : 0) << 32);
  cqlcuda_kernel_set_arg_u64(kflags, 4, (uint64_t)(key_count > 2 ? keys[2].base : 0) | (uint64_t)(key_count > 3 ? keys[3].base : 0) << 32);
  cqlcuda_batch_kernel_execute(b, kflags, (uint32_t)n, QE_GPU_WORKGROUP_SIZE);
  cqlcuda_kernel_set_arg_buffer(ktiles, 0, flags);
  cqlcuda_kernel_set_arg_buffer(ktiles, 1, agg);
  cqlcuda_kernel_set_arg_u64(ktiles, 0, n);
  cqlcuda_batch_kernel_execute(b, ktiles, (uint32_t)(tiles * QE_GPU_WORKGROUP_SIZE), QE_GPU_WORKGROUP_SIZE);
  cqlcuda_kernel_set_arg_buffer(kcarry, 0, agg);
  cqlcuda_kernel_set_arg_buffer(kcarry, 1, carry);
  cqlcuda_kernel_set_arg_u64(kcarry, 0, tiles);
  cqlcuda_batch_kernel_execute(b, kcarry, QE_GPU_WORKGROUP_SIZE, QE_GPU_WORKGROUP_SIZE);
  cqlcuda_kernel_set_arg_buffer(kapply, 0, flags);
  cqlcuda_kernel_set_arg_buffer(kapply, 1, carry);
  cqlcuda_kernel_set_arg_buffer_range(kapply, 2, ranks, 0, n * 4);
  cqlcuda_kernel_set_arg_buffer_range(kapply, 3, ranks, n * 4, n * 4);
  cqlcuda_kernel_set_arg_buffer_range(kapply, 4, ranks, n * 8, n * 4);
  cqlcuda_kernel_set_arg_u64(kapply, 0, n);
  cqlcuda_batch_kernel_execute(b, kapply, (uint32_t)(tiles * QE_GPU_WORKGROUP_SIZE), QE_GPU_WORKGROUP_SIZE);
  if (out_rows) cqlcuda_batch_buffer_read(b, sorted, out_rows, n * 4);
  if (out_row_number) cqlcuda_batch_buffer_read_at(b, ranks, 0, out_row_number, n * 4);
  if (out_rank) cqlcuda_batch_buffer_read_at(b, ranks, n * 4, out_rank, n * 4);
  if (out_dense_rank) cqlcuda_batch_buffer_read_at(b, ranks, n * 8, out_dense_rank, n * 4);
  return cqlcuda_batch_end(b);
}
