/*
 * cql_ops.c - C99 operator layer: drives the cqlcuda backend with the reference operator layer's
 * kernels, bindings, push-constant words and host folds (src/query_exec/query_exec.c), on whole
 * device-resident columns.
 */
#include "cqlops.h"
#include "cql_ops_internal.h"

#include <math.h>
#include <stdio.h>
#include <stdlib.h>
#include <string.h>

#define QE_GPU_WORKGROUP_SIZE 256
#define QE_AGG_STREAM_DEFAULT_GROUPS 2048
#define QE_AGG_STREAM_MAX_COLUMNS 4
#define QE_SIMPLE_SCAN_MAX_LEAVES 8
#define SCAN_MAX_RANGES 64
#define QE_SIMPLE_SCAN_ROWS_PER_THREAD 8
#define QE_MAX_COLUMN_BINDINGS 10
#define QE_DENSE_STREAM_MAX_ARGS 4
#define QE_DENSE_STREAM_MAX_GROUPS 65536
#define QE_DENSE_STREAM_ACC_WORDS 2048
#define QE_DENSE_STREAM_MM_WORDS 1024
#define QE_DENSE_STREAM_MAX_TILES 256
#define QE_AGG_MAX_EXPRS 8
#define QE_F64_MAX 1.7976931348623157e308

#define QE_SCAN_INT_FLAG  0x10000u
#define QE_SCAN_INT_NEVER 0x20000u
#define QE_SCAN_INT_BIAS  0x40000u

/* per calling thread: operators run concurrently on threads with their own backend lanes */
static __thread uint32_t g_launch_mark = 0;
static __thread char g_error[256] = "";

const char* cqlops_last_error(void)
{
  return g_error;
}

/* Records why a request is refused (the reference logs and returns 0 at the same points). */
void cqlops_note_error(const char* why)
{
  snprintf(g_error, sizeof(g_error), "%s", why);
  /* an operator starting afresh also drops the backend's text of an earlier failure */
  if (!why[0]) cqlcuda_clear_error();
}

static int refuse(const char* why)
{
  cqlops_note_error(why);
  return 0;
}

/* Row numbers and row counts reach the kernels as 32-bit push-constant words (the reference's shaders
   take them the same way; its operators never pass more than a 16M-row chunk). A column of more
   rows is refused before any device work rather than truncated. */
int cqlops_rows_fit(uint64_t rows)
{
  if (rows <= CQLOPS_MAX_ROWS) return 1;
  char why[200];
  snprintf(why, sizeof(why), "%llu rows: an operator takes at most %llu rows (32-bit row numbers); run it over slices of the table",
           (unsigned long long)rows, (unsigned long long)CQLOPS_MAX_ROWS);
  cqlops_note_error(why);
  return 0;
}

uint32_t cqlops_last_launches(void)
{
  return cqlcuda_kernel_launch_count() - g_launch_mark;
}

static void launches_begin(void)
{
  g_launch_mark = cqlcuda_kernel_launch_count();
  cqlops_note_error("");
}

static CqlKernel* kernel_named(const char* name)
{
  return cqlcuda_kernel_alloc(name, (uint64_t)strlen(name));
}

static CqlBuffer* pooled(const char* name, uint64_t size, uint32_t flags)
{
  return cqlcuda_buffer_alloc_pooled(name, (uint64_t)strlen(name), size, flags, NULL);
}

/* A column the kernels read as `width` bytes per row (qe_encoding_shader_width, query_exec.c:1593-1601). */
static uint32_t shader_width(const CqlColumn* c)
{
  return c->width == 4 ? 0u : c->width;
}

/* ------------------------------------------------------------------------------------------------
 * SUM / MIN / MAX of whole columns: qe_aggregate_global_streamed (query_exec.c:8842-9112) */

/* The workgroup partials folded, in workgroup order, into running totals that start at io_* (reset: at
   0, +F64_MAX and -F64_MAX, qe_agg_stream_begin) */
static int aggregate_global_fold(const CqlColumn* columns, uint32_t column_count, double* io_sum, double* io_min, double* io_max, int reset);

int cqlops_aggregate_global(const CqlColumn* columns, uint32_t column_count, double* out_sum, double* out_min, double* out_max)
{
  return aggregate_global_fold(columns, column_count, out_sum, out_min, out_max, 1);
}

int cqlops_aggregate_global_accumulate(const CqlColumn* columns, uint32_t column_count, double* io_sum, double* io_min, double* io_max)
{
  if (!io_sum || !io_min || !io_max) return refuse("the running totals are required");
  return aggregate_global_fold(columns, column_count, io_sum, io_min, io_max, 0);
}

static int aggregate_global_fold(const CqlColumn* columns, uint32_t column_count, double* out_sum, double* out_min, double* out_max, int reset)
{
  launches_begin();
  if (column_count == 0 || column_count > QE_AGG_STREAM_MAX_COLUMNS)
  {
    return 0;
  }
  uint64_t rows = columns[0].rows;
  for (uint32_t c = 0; c < column_count; c++)
    if (!cqlops_rows_fit(columns[c].rows)) return 0;
  double sum[QE_AGG_STREAM_MAX_COLUMNS], mn[QE_AGG_STREAM_MAX_COLUMNS], mx[QE_AGG_STREAM_MAX_COLUMNS];
  const CqlColumn* gpu_cols[QE_AGG_STREAM_MAX_COLUMNS];
  uint32_t gpu_to_col[QE_AGG_STREAM_MAX_COLUMNS];
  uint32_t gpu_count = 0;
  for (uint32_t c = 0; c < column_count; c++)
  {
    const CqlColumn* col = &columns[c];
    uint32_t t = col->type;
    if (col->rows != rows || !(t == CQLOPS_TYPE_U32 || t == CQLOPS_TYPE_I32 || t == CQLOPS_TYPE_F32 || t == CQLOPS_TYPE_F64))
    {
      return 0;
    }
    sum[c] = reset ? 0.0 : out_sum[c];
    mn[c] = reset ? QE_F64_MAX : out_min[c];
    mx[c] = reset ? -QE_F64_MAX : out_max[c];
    if (col->width == 3)
    {
      /* base + row number: n * first + n * (n - 1) / 2 in 64-bit whole numbers, rounded once (:8906-8916) */
      int64_t first = t == CQLOPS_TYPE_I32 ? (int64_t)(int32_t)col->base : (int64_t)col->base;
      uint64_t n = rows;
      if (n > 0)
      {
        int64_t total = first * (int64_t)n + (int64_t)(n * (n - 1) / 2);
        sum[c] += (double)total;
        mn[c] = (double)first < mn[c] ? (double)first : mn[c];
        mx[c] = (double)first + (double)(n - 1) > mx[c] ? (double)first + (double)(n - 1) : mx[c];
      }
    }
    else
    {
      if (!col->buffer)
      {
        return 0;
      }
      gpu_cols[gpu_count] = col;
      gpu_to_col[gpu_count] = c;
      gpu_count++;
    }
  }
  if (gpu_count > 0 && rows > 0)
  {
    CqlKernel* k = kernel_named("aggregate_global_native");
    if (!k)
    {
      return 0;
    }
    uint64_t group_count = QE_AGG_STREAM_DEFAULT_GROUPS;
    uint64_t partial_count = group_count * gpu_count * 3;
    CqlBuffer* partials_buf = pooled("cqlops_agg_global_partials", partial_count * sizeof(double), CQLCUDA_BUFFER_READ);
    double* partials = (double*)malloc(partial_count * sizeof(double));
    if (!partials_buf || !partials)
    {
      free(partials);
      return 0;
    }
    /* a binding with no column behind it is bound to the first column; the kernel never reads it */
    for (uint32_t b = 0; b < QE_AGG_STREAM_MAX_COLUMNS; b++)
    {
      cqlcuda_kernel_set_arg_buffer(k, b, gpu_cols[b < gpu_count ? b : 0]->buffer);
    }
    cqlcuda_kernel_set_arg_buffer(k, QE_AGG_STREAM_MAX_COLUMNS, partials_buf);
    cqlcuda_kernel_set_arg_u64(k, 0, rows);
    cqlcuda_kernel_set_arg_u64(k, 1, gpu_count);
    cqlcuda_kernel_set_arg_u64(k, 2, group_count);
    for (uint32_t c = 0; c < QE_AGG_STREAM_MAX_COLUMNS; c++)
    {
      uint64_t type_word = 0;
      if (c < gpu_count)
      {
        type_word = (uint64_t)gpu_cols[c]->type | ((uint64_t)shader_width(gpu_cols[c]) << 8) | ((uint64_t)gpu_cols[c]->base << 32);
      }
      cqlcuda_kernel_set_arg_u64(k, 3 + c, type_word);
    }
    CqlBatch* batch = cqlcuda_batch_begin(0, partial_count * sizeof(double));
    cqlcuda_batch_kernel_execute(batch, k, (uint32_t)(group_count * QE_GPU_WORKGROUP_SIZE), QE_GPU_WORKGROUP_SIZE);
    cqlcuda_batch_buffer_read(batch, partials_buf, partials, partial_count * sizeof(double));
    if (!cqlcuda_batch_end(batch))
    {
      free(partials);
      return 0;
    }
    /* folded in workgroup order (qe_agg_stream_retire, :8812-8841) */
    for (uint64_t g = 0; g < group_count; g++)
    {
      for (uint32_t c = 0; c < gpu_count; c++)
      {
        const double* triple = &partials[(g * gpu_count + c) * 3];
        uint32_t dst = gpu_to_col[c];
        sum[dst] += triple[0];
        mn[dst] = triple[1] < mn[dst] ? triple[1] : mn[dst];
        mx[dst] = triple[2] > mx[dst] ? triple[2] : mx[dst];
      }
    }
    free(partials);
  }
  for (uint32_t c = 0; c < column_count; c++)
  {
    if (out_sum) out_sum[c] = sum[c];
    if (out_min) out_min[c] = mn[c];
    if (out_max) out_max[c] = mx[c];
  }
  return 1;
}

/* ------------------------------------------------------------------------------------------------
 * scan_simple leaves: qe_scan_int_interval / qe_scan_int_leaf_words / qe_simple_leaf_words
 * (query_exec.c:1378-1460), and the narrow rewrite of qe_scan_filter_streamed (:2294-2321). */

static int scan_int_interval(uint32_t op, double target, double code_offset, double max_code, uint32_t* out_lo, uint32_t* out_span)
{
  if (target != target)
  {
    return 0;
  }
  double low = -1e18;
  double high = 1e18;
  switch (op)
  {
    case 0:
      if (floor(target) != target) return 0;
      low = target;
      high = target;
      break;
    case 1: high = ceil(target) - 1.0; break;
    case 2: high = floor(target); break;
    case 3: low = floor(target) + 1.0; break;
    case 4: low = ceil(target); break;
    default: return 0;
  }
  low = low - code_offset;
  if (low < 0.0) low = 0.0;
  high = high - code_offset;
  if (high > max_code) high = max_code;
  if (low > high)
  {
    return 0;
  }
  *out_lo = (uint32_t)low;
  *out_span = (uint32_t)(high - low);
  return 1;
}

static void scan_int_leaf_words(uint32_t* words, uint32_t type, uint32_t op, double target, uint32_t width, uint32_t base)
{
  double code_offset = 0.0;
  double max_code = 4294967295.0;
  uint32_t flags = QE_SCAN_INT_FLAG;
  if (width == 3)
  {
    code_offset = type == CQLOPS_TYPE_I32 ? (double)(int32_t)base : (double)base;
  }
  else if (width == 1 || width == 2)
  {
    max_code = width == 1 ? 255.0 : 65535.0;
    code_offset = type == CQLOPS_TYPE_I32 ? (double)(int32_t)base : (double)base;
  }
  else if (type == CQLOPS_TYPE_I32)
  {
    code_offset = -2147483648.0;
    flags |= QE_SCAN_INT_BIAS;
  }
  uint32_t lo = 0, span = 0;
  if (!scan_int_interval(op, target, code_offset, max_code, &lo, &span))
  {
    flags |= QE_SCAN_INT_NEVER;
  }
  words[1] = type | (width << 8) | flags;
  words[3] = lo;
  words[4] = span;
  words[5] = 0;
}

static int simple_leaf_words(uint32_t* words, uint32_t slot, const CqlColumn* col, uint32_t op, double target)
{
  uint64_t bits;
  memcpy(&bits, &target, sizeof(bits));
  words[0] = slot;
  words[1] = col->type;
  words[2] = op;
  words[3] = (uint32_t)(bits & 0xffffffffu);
  words[4] = (uint32_t)(bits >> 32);
  words[5] = 0;
  uint32_t w = shader_width(col);
  if (col->type == CQLOPS_TYPE_U32 || col->type == CQLOPS_TYPE_I32)
  {
    scan_int_leaf_words(words, col->type, op, target, w, col->base);
  }
  else if (w != 0)
  {
    return 0; /* narrow or sequence encodings exist only for whole-number columns */
  }
  return 1;
}

/* The rows of a selection bitmap (one bit a row, as the scans write it in bitmap mode; its first bit is
   table row first_row, a multiple of 32) in ascending order, on the device: each 256-word block's
   population, an exclusive scan over the blocks, then every block's rows written from its offset. The
   first min(count, cap) rows land in out_rows; count is the bitmap's population. */
/* Enqueues into batch b the rows of a selection bitmap of `rows` rows, ascending, into `list` (at most its
   size / 4 of them; the emit kernel stops there). */
int cqlops_bitmap_rows_enqueue(CqlBatch* b, CqlBuffer* bitmap, uint64_t first_row, uint64_t rows, CqlBuffer* list)
{
  uint64_t words = (rows + 31) / 32, blocks = (words + 255) / 256, scan_blocks = (blocks + 255) / 256;
  if (words == 0) return 1;
  CqlBuffer* counts = pooled("bitmap_block_counts", blocks * 4, CQLCUDA_BUFFER_READ_WRITE);
  CqlBuffer* offsets = pooled("bitmap_block_offsets", (blocks + 1) * 4, CQLCUDA_BUFFER_READ_WRITE);
  CqlBuffer* cursor = pooled("bitmap_block_cursor", blocks * 4, CQLCUDA_BUFFER_READ_WRITE);
  CqlBuffer* block_sums = pooled("bitmap_scan_sums", scan_blocks * 4, CQLCUDA_BUFFER_READ_WRITE);
  CqlKernel* popc = kernel_named("cql_bitmap_popc");
  CqlKernel* scan = kernel_named("prefix_sum");
  CqlKernel* emit = kernel_named("cql_bitmap_emit");
  if (!counts || !offsets || !cursor || !block_sums || !popc || !scan || !emit) return 0;
  cqlcuda_kernel_set_arg_buffer(popc, 0, bitmap);
  cqlcuda_kernel_set_arg_buffer(popc, 1, counts);
  cqlcuda_kernel_set_arg_u64(popc, 0, words);
  cqlcuda_kernel_set_arg_buffer(scan, 0, counts);
  cqlcuda_kernel_set_arg_buffer(scan, 1, offsets);
  cqlcuda_kernel_set_arg_buffer(scan, 2, cursor);
  cqlcuda_kernel_set_arg_buffer(scan, 3, block_sums);
  cqlcuda_kernel_set_arg_u64(scan, 0, blocks);
  cqlcuda_kernel_set_arg_buffer(emit, 0, bitmap);
  cqlcuda_kernel_set_arg_buffer(emit, 1, offsets);
  cqlcuda_kernel_set_arg_buffer(emit, 2, list);
  cqlcuda_kernel_set_arg_u64(emit, 0, words);
  cqlcuda_kernel_set_arg_u64(emit, 1, first_row);
  if (blocks == 1) cqlcuda_batch_buffer_zero(b, offsets, 4);   /* one block: its rows start at 0 */
  else
  {
    cqlcuda_batch_kernel_execute(b, popc, (uint32_t)(blocks * 256), QE_GPU_WORKGROUP_SIZE);
    for (uint32_t mode = 0; mode < 3; mode++)
    {
      cqlcuda_kernel_set_arg_u64(scan, 1, mode);
      cqlcuda_batch_kernel_execute(b, scan, mode == 1 ? 256u : (uint32_t)(scan_blocks * 256), 256);
    }
  }
  cqlcuda_batch_kernel_execute(b, emit, (uint32_t)(blocks * 256), QE_GPU_WORKGROUP_SIZE);
  return 1;
}

/* The rows of a selection bitmap (one bit a row, as the scans write it in bitmap mode; its first bit is
   table row first_row, a multiple of 32) in ascending order, on the device: each 256-word block's
   population, an exclusive scan over the blocks, then every block's rows written from its offset. The
   first min(count, cap) rows land in out_rows; count is the bitmap's population. */
int cqlops_bitmap_rows(CqlBuffer* bitmap, uint64_t first_row, uint64_t rows, uint64_t count, uint32_t* out_rows, uint64_t cap)
{
  if (!count || !cap || !out_rows) return 1;
  uint64_t n = count < cap ? count : cap;
  CqlBuffer* list = pooled("bitmap_rows", n * 4, CQLCUDA_BUFFER_READ_WRITE);
  if (!list) return 0;
  CqlBatch* b = cqlcuda_batch_begin(0, n * 4);
  if (!cqlops_bitmap_rows_enqueue(b, bitmap, first_row, rows, list))
  {
    cqlcuda_batch_end(b);
    return 0;
  }
  cqlcuda_batch_buffer_read(b, list, out_rows, n * 4);
  return cqlcuda_batch_end(b);
}

static int scan_simple_run(const CqlColumn* columns, uint32_t column_count, const CqlLeaf* leaves, uint32_t leaf_count, uint64_t* out_count,
                           uint32_t* out_rows, uint64_t out_capacity, CqlBuffer* out_selection)
{
  launches_begin();
  if (leaf_count == 0 || leaf_count > QE_SIMPLE_SCAN_MAX_LEAVES || column_count == 0 || column_count > QE_MAX_COLUMN_BINDINGS)
  {
    return 0;
  }
  uint64_t rows = columns[0].rows;
  for (uint32_t c = 0; c < column_count; c++)
    if (!cqlops_rows_fit(columns[c].rows)) return 0;
  uint32_t words[1 + QE_SIMPLE_SCAN_MAX_LEAVES * 6];
  memset(words, 0, sizeof(words));
  words[0] = leaf_count;
  for (uint32_t l = 0; l < leaf_count; l++)
  {
    if (leaves[l].column >= column_count)
    {
      return 0;
    }
    const CqlColumn* col = &columns[leaves[l].column];
    uint32_t t = col->type;
    if (col->rows != rows || !(t == CQLOPS_TYPE_U32 || t == CQLOPS_TYPE_I32 || t == CQLOPS_TYPE_F32 || t == CQLOPS_TYPE_F64))
    {
      return 0;
    }
    if (!simple_leaf_words(&words[1 + l * 6], leaves[l].column, col, leaves[l].op, leaves[l].target))
    {
      return 0;
    }
  }
  if (rows == 0)
  {
    /* an empty table matches nothing: no device work */
    if (out_count) *out_count = 0;
    return 1;
  }
  CqlKernel* k = kernel_named("scan_simple");
  if (!k)
  {
    return 0;
  }
  CqlBuffer* leaf_buf = pooled("cqlops_scan_leaves", sizeof(words), CQLCUDA_BUFFER_WRITE);
  CqlBuffer* counter = pooled("scan_filter_result_counter", 2 * sizeof(uint32_t), CQLCUDA_BUFFER_READ_WRITE);
  if (!leaf_buf || !counter)
  {
    return 0;
  }
  /* the output: none for a count, else a bitmap of the rows (no capacity to outgrow, unlike the
     reference's list sized at :3084-3090) */
  int want_rows = out_rows != NULL || out_selection != NULL;
  /* zone-map pruning: the ranges of the table the leaves can match, or one pass with a skip bitmap
     (qe_scan_build_dispatch_ranges, :13307-13540) */
  uint64_t chunks = (rows + CQLOPS_ZONEMAP_CHUNK_ROWS - 1) / CQLOPS_ZONEMAP_CHUNK_ROWS;
  uint64_t ranges[2 * SCAN_MAX_RANGES];
  uint32_t* skip_bits = (uint32_t*)malloc(((chunks + 31) / 32 + 1) * sizeof(uint32_t));
  int use_skip = 0;
  uint64_t pruned_rows = 0;
  if (!skip_bits) return 0;
  uint64_t range_count = cqlops_scan_ranges(columns, column_count, leaves, leaf_count, ranges, SCAN_MAX_RANGES, skip_bits, &use_skip,
                                            &pruned_rows);
  CqlBuffer* skip_buf = counter; /* the skip binding always holds a buffer; it only counts when enabled */
  if (use_skip)
  {
    skip_buf = pooled("scan_filter_skip", ((chunks + 31) / 32) * sizeof(uint32_t), CQLCUDA_BUFFER_WRITE);
    if (!skip_buf)
    {
      free(skip_bits);
      return 0;
    }
  }
  cqlcuda_kernel_set_arg_buffer(k, 0, leaf_buf);
  cqlcuda_kernel_set_arg_buffer(k, 4, counter);
  cqlcuda_kernel_set_arg_buffer(k, 5, skip_buf);
  cqlcuda_kernel_set_arg_u64(k, 3, use_skip ? 13 : 0);
  cqlcuda_kernel_set_arg_u64(k, 4, use_skip ? 1 : 0);
  /* the matches as a bitmap of the rows from the first range's start to the last range's end (word 14;
     word 2 its first row), turned into ascending rows on the device */
  uint64_t bitmap_first = range_count ? ranges[0] : 0, bitmap_end = range_count ? ranges[2 * range_count - 1] : 0;
  uint64_t bitmap_words = (bitmap_end - bitmap_first + 31) / 32;
  CqlBuffer* output = want_rows ? pooled("scan_bitmap", (bitmap_words ? bitmap_words : 1) * 4, CQLCUDA_BUFFER_READ_WRITE)
                                : pooled("cqlops_scan_no_output", 0, CQLCUDA_BUFFER_READ);   /* count only */
  if (!output)
  {
    free(skip_bits);
    return 0;
  }
  cqlcuda_kernel_set_arg_buffer(k, 3, output);
  cqlcuda_kernel_set_arg_u64(k, 7, want_rows ? 1 : 0);
  cqlcuda_kernel_set_arg_u64(k, 1, bitmap_first);
  uint32_t count32[2] = { 0, 0 };
  CqlBatch* batch = cqlcuda_batch_begin(sizeof(words) + (use_skip ? ((chunks + 31) / 32) * 4 : 0), sizeof(count32));
  cqlcuda_batch_buffer_write(batch, leaf_buf, words, sizeof(words));
  if (use_skip) cqlcuda_batch_buffer_write(batch, skip_buf, skip_bits, ((chunks + 31) / 32) * sizeof(uint32_t));
  cqlcuda_batch_buffer_zero(batch, counter, sizeof(count32));
  /* ranges a zone map keeps leave the words between them unwritten: they must read as no match */
  if (want_rows && range_count > 1) cqlcuda_batch_buffer_zero(batch, output, bitmap_words * 4);
  for (uint64_t r = 0; r < range_count; r++)
  {
    /* one dispatch per range: the columns bound from the range's first row, row numbers written
       from there (a sequence column's values from chunk_start) */
    uint64_t start = ranges[2 * r], end = ranges[2 * r + 1];
    for (uint32_t c = 0; c < QE_MAX_COLUMN_BINDINGS; c++)
    {
      const CqlColumn* col = &columns[c < column_count ? c : 0];
      if (!col->buffer)
      {
        cqlcuda_kernel_set_arg_buffer(k, 6 + c, leaf_buf); /* a sequence column is never read */
        continue;
      }
      uint64_t elem = col->width == 1 ? 1 : col->width == 2 ? 2 : col->type == CQLOPS_TYPE_F64 ? 8 : 4;
      uint64_t size = cqlcuda_buffer_size(col->buffer);
      uint64_t offset = start * elem;
      cqlcuda_kernel_set_arg_buffer_range(k, 6 + c, col->buffer, offset, size > offset ? size - offset : 0);
    }
    cqlcuda_kernel_set_arg_u64(k, 0, end - start);
    cqlcuda_kernel_set_arg_u64(k, 5, start);
    cqlcuda_kernel_set_arg_u64(k, 6, start);
    uint64_t threads = (end - start + QE_SIMPLE_SCAN_ROWS_PER_THREAD - 1) / QE_SIMPLE_SCAN_ROWS_PER_THREAD;
    cqlcuda_batch_kernel_execute(batch, k, (uint32_t)threads, QE_GPU_WORKGROUP_SIZE);
  }
  /* a device selection: the rows are listed in the same batch (the list stops at the buffer's size) */
  if (out_selection && !cqlops_bitmap_rows_enqueue(batch, output, bitmap_first, bitmap_end - bitmap_first, out_selection))
  {
    cqlcuda_batch_end(batch);
    free(skip_bits);
    return 0;
  }
  cqlcuda_batch_buffer_read(batch, counter, count32, sizeof(count32));
  if (!cqlcuda_batch_end(batch))
  {
    free(skip_bits);
    return 0;
  }
  uint64_t result_count = count32[0];
  free(skip_bits);
  if (out_rows && !cqlops_bitmap_rows(output, bitmap_first, bitmap_end - bitmap_first, result_count, out_rows, out_capacity)) return 0;
  if (out_count) *out_count = result_count;
  return 1;
}

int cqlops_scan_simple(const CqlColumn* columns, uint32_t column_count, const CqlLeaf* leaves, uint32_t leaf_count, uint64_t* out_count,
                       uint32_t* out_rows, uint64_t out_capacity)
{
  return scan_simple_run(columns, column_count, leaves, leaf_count, out_count, out_rows, out_capacity, NULL);
}

int cqlops_scan_simple_select(const CqlColumn* columns, uint32_t column_count, const CqlLeaf* leaves, uint32_t leaf_count,
                              CqlBuffer* out_selection, uint64_t* out_count)
{
  if (!out_selection) return refuse("a device buffer for the selection");
  return scan_simple_run(columns, column_count, leaves, leaf_count, out_count, NULL, 0, out_selection);
}

/* ------------------------------------------------------------------------------------------------
 * Dense GROUP BY: qe_dense_stream_core (query_exec.c:7632-7983) on one chunk */

static int group_dense_run(const CqlColumn* key, uint64_t rows, uint32_t expr_count, const uint32_t* funcs, const CqlColumn* const* arg_cols,
                           uint64_t max_groups, uint64_t* out_group_count, int64_t* out_min_key, uint64_t* out_counts, int64_t* out_sums,
                           int64_t* out_mins, int64_t* out_maxs, CqlDenseTotals* device_out);

int cqlops_group_dense(const CqlColumn* key, uint64_t rows, uint32_t expr_count, const uint32_t* funcs, const CqlColumn* const* arg_cols,
                       uint64_t max_groups, uint64_t* out_group_count, int64_t* out_min_key, uint64_t* out_counts, int64_t* out_sums,
                       int64_t* out_mins, int64_t* out_maxs)
{
  return group_dense_run(key, rows, expr_count, funcs, arg_cols, max_groups, out_group_count, out_min_key, out_counts, out_sums, out_mins,
                         out_maxs, NULL);
}

/* the dense group-by with its totals kept in its pooled device buffer (the join's device dim-row pass) */
int cql_group_dense_device(const CqlColumn* key, uint64_t rows, uint32_t expr_count, const uint32_t* funcs, const CqlColumn* const* arg_cols,
                           uint64_t max_groups, CqlDenseTotals* out)
{
  return group_dense_run(key, rows, expr_count, funcs, arg_cols, max_groups, NULL, NULL, NULL, NULL, NULL, NULL, out);
}

static int group_dense_run(const CqlColumn* key, uint64_t rows, uint32_t expr_count, const uint32_t* funcs, const CqlColumn* const* arg_cols,
                           uint64_t max_groups, uint64_t* out_group_count, int64_t* out_min_key, uint64_t* out_counts, int64_t* out_sums,
                           int64_t* out_mins, int64_t* out_maxs, CqlDenseTotals* device_out)
{
  launches_begin();
  if (!cqlops_rows_fit(rows)) return 0;
  if (rows == 0 && !device_out && key && key->rows == 0)
  {
    /* an empty table has no groups (no device work) */
    if (out_group_count) *out_group_count = 0;
    if (out_min_key) *out_min_key = 0;
    return 1;
  }
  /* a dictionary string column groups by its codes, as the reference's dictionary GROUP BY does */
  int dict_key = key && key->type == CQLOPS_TYPE_STRING8 && key->dict && key->width == 0;
  if (!key || !key->has_range || !(key->type == CQLOPS_TYPE_U32 || key->type == CQLOPS_TYPE_I32 || dict_key) || key->rows != rows || !key->buffer ||
      key->width == 3 || key->zone_min < -2147483648.0 || key->zone_max > 2147483647.0 ||
      key->zone_max - key->zone_min + 1.0 > (double)QE_DENSE_STREAM_MAX_GROUPS)
  {
    return refuse("dense group-by: the key must be a whole-number or dictionary string column with a zone range of at most 65536 values");
  }
  int64_t min_key = (int64_t)key->zone_min;
  uint64_t group_count = (uint64_t)((int64_t)key->zone_max - min_key) + 1;
  if (group_count > max_groups || expr_count == 0 || expr_count > QE_AGG_MAX_EXPRS)
  {
    return 0;
  }
  const CqlColumn* arg_columns[QE_DENSE_STREAM_MAX_ARGS] = { 0 };
  uint32_t arg_count = 0, func_codes = 0, arg_index_codes = 0, arg_signed_bits = 0;
  double largest_sum_arg = 0.0;
  int has_min_max = 0;
  for (uint32_t e = 0; e < expr_count; e++)
  {
    uint32_t f = funcs[e];
    if (f > CQLOPS_FUNC_MAX)
    {
      return 0;
    }
    func_codes |= (f & 0xfu) << (e * 4u);
    if (f == CQLOPS_FUNC_COUNT)
    {
      continue;
    }
    const CqlColumn* col = arg_cols[e];
    if (!col || !(col->type == CQLOPS_TYPE_U32 || col->type == CQLOPS_TYPE_I32) || col->rows != rows || (!col->buffer && col->width != 3))
    {
      return 0;
    }
    /* MIN and MAX are signed 32-bit atomics, so the values have to fit (:7712-7718) */
    if ((f == CQLOPS_FUNC_MIN || f == CQLOPS_FUNC_MAX) && (!col->has_range || col->zone_min < -2147483648.0 || col->zone_max > 2147483647.0))
    {
      return refuse("dense group-by: MIN/MAX values must fit a signed 32-bit word");
    }
    if (f == CQLOPS_FUNC_MIN || f == CQLOPS_FUNC_MAX) has_min_max = 1;
    if (f == CQLOPS_FUNC_SUM || f == CQLOPS_FUNC_AVG)
    {
      double m = col->has_range ? (col->zone_max > -col->zone_min ? col->zone_max : -col->zone_min) : 4294967296.0;
      if (m > largest_sum_arg) largest_sum_arg = m;
    }
    uint32_t index = 0;
    while (index < arg_count && arg_columns[index] != col) index++;
    if (index == arg_count)
    {
      if (arg_count == QE_DENSE_STREAM_MAX_ARGS) return 0;
      arg_columns[arg_count++] = col;
    }
    arg_index_codes |= (index & 0xfu) << (e * 4u);
    if (col->type == CQLOPS_TYPE_I32) arg_signed_bits |= 1u << index;
  }
  uint64_t slice_rows = 16384;
  int narrow_sums = largest_sum_arg * (double)slice_rows < 1073741824.0;
  uint64_t acc_stride = (1 + (narrow_sums ? 1 : 2) * (uint64_t)expr_count) | 1;
  uint64_t mm_stride = has_min_max ? (2 * (uint64_t)expr_count) | 1 : 0;
  uint64_t tile_groups = QE_DENSE_STREAM_ACC_WORDS / acc_stride;
  if (mm_stride && QE_DENSE_STREAM_MM_WORDS / mm_stride < tile_groups) tile_groups = QE_DENSE_STREAM_MM_WORDS / mm_stride;
  if (tile_groups > group_count) tile_groups = group_count;
  uint64_t tile_count = (group_count + tile_groups - 1) / tile_groups;
  if (tile_count > QE_DENSE_STREAM_MAX_TILES)
  {
    return refuse("dense group-by: more than 256 tiles of the reference's shared-memory slices");
  }
  CqlKernel* k = kernel_named("aggregate_dense_native");
  if (!k)
  {
    return 0;
  }
  /* the key's encoding base must be the smallest key (:7778-7781) */
  uint64_t key_width = shader_width(key);
  if ((key_width == 1 || key_width == 2) && key->base != (uint32_t)(int32_t)min_key)
  {
    return 0;
  }
  uint64_t shader_widths = key_width;
  uint32_t arg_bases[QE_DENSE_STREAM_MAX_ARGS] = { 0 };
  for (uint32_t i = 0; i < arg_count; i++)
  {
    shader_widths |= (uint64_t)shader_width(arg_columns[i]) << (4 + 4 * i);
    arg_bases[i] = arg_columns[i]->base;
  }
  uint64_t info_bytes = group_count * 2 * sizeof(uint32_t);
  uint64_t sum_bytes = group_count * expr_count * 2 * sizeof(uint32_t);
  uint64_t mm_bytes = group_count * expr_count * sizeof(uint32_t);
  /* the four outputs in one buffer (info, sums, then MIN and MAX words, each part 16-byte aligned), bound
     as four ranges: one clear and one read-back for the counts and sums */
  uint64_t sum_at = (info_bytes + 15) & ~15ull;
  uint64_t min_at = (sum_at + sum_bytes + 15) & ~15ull;
  uint64_t max_at = (min_at + mm_bytes + 15) & ~15ull;
  uint64_t out_bytes = max_at + mm_bytes;
  CqlBuffer* out_buf = pooled("cqlops_dense_out", out_bytes, CQLCUDA_BUFFER_READ_WRITE);
  unsigned char* host_out = (unsigned char*)malloc(out_bytes);
  uint32_t* info = (uint32_t*)host_out;
  uint32_t* sums = host_out ? (uint32_t*)(host_out + sum_at) : NULL;
  uint32_t* mins = host_out ? (uint32_t*)(host_out + min_at) : NULL;
  uint32_t* maxs = host_out ? (uint32_t*)(host_out + max_at) : NULL;
  int ok = out_buf && host_out;
  if (ok)
  {
    cqlcuda_kernel_set_arg_buffer(k, 0, key->buffer);
    for (uint32_t b = 0; b < QE_DENSE_STREAM_MAX_ARGS; b++)
    {
      const CqlColumn* col = b < arg_count ? arg_columns[b] : key;
      cqlcuda_kernel_set_arg_buffer(k, 1 + b, col->buffer ? col->buffer : key->buffer);
    }
    cqlcuda_kernel_set_arg_buffer_range(k, 5, out_buf, 0, info_bytes);
    cqlcuda_kernel_set_arg_buffer_range(k, 6, out_buf, sum_at, sum_bytes);
    cqlcuda_kernel_set_arg_buffer_range(k, 7, out_buf, min_at, mm_bytes);
    cqlcuda_kernel_set_arg_buffer_range(k, 8, out_buf, max_at, mm_bytes);
    cqlcuda_kernel_set_arg_u64(k, 0, rows | (shader_widths << 32));
    cqlcuda_kernel_set_arg_u64(k, 1, (uint64_t)expr_count | ((uint64_t)arg_bases[0] << 32));
    cqlcuda_kernel_set_arg_u64(k, 2, (uint64_t)func_codes | ((uint64_t)arg_bases[1] << 32));
    cqlcuda_kernel_set_arg_u64(k, 3, (uint64_t)arg_index_codes | ((uint64_t)(arg_signed_bits | (narrow_sums ? 0x80000000u : 0u)) << 32));
    cqlcuda_kernel_set_arg_u64(k, 4, group_count | ((uint64_t)arg_bases[2] << 32));
    cqlcuda_kernel_set_arg_u64(k, 5, (uint64_t)(uint32_t)(int32_t)min_key | ((uint64_t)arg_bases[3] << 32));
    cqlcuda_kernel_set_arg_u64(k, 6, tile_groups | (slice_rows << 32));
    cqlcuda_kernel_set_arg_u64(k, 7, tile_count);
    /* the kernel touches the MIN/MAX arrays only for MIN/MAX expressions: without any, their initial
       values are the results and neither array crosses the bus */
    uint64_t counted = has_min_max ? out_bytes : min_at;
    CqlBatch* batch = cqlcuda_batch_begin(0, device_out ? 0 : counted);
    cqlcuda_batch_buffer_zero(batch, out_buf, min_at);
    if (has_min_max || device_out)
    {
      cqlcuda_batch_fill_range(batch, out_buf, min_at, mm_bytes, 0x7fffffffu);
      cqlcuda_batch_fill_range(batch, out_buf, max_at, mm_bytes, 0x80000000u);
    }
    uint64_t workgroups = (rows + slice_rows - 1) / slice_rows;
    cqlcuda_batch_kernel_execute(batch, k, (uint32_t)(workgroups * QE_GPU_WORKGROUP_SIZE), QE_GPU_WORKGROUP_SIZE);
    if (device_out)
    {
      /* the totals stay on the device for the caller's next operations: in this batch, left open (no wait
         between the two), or in a batch of its own */
      device_out->batch = NULL;
      if (device_out->keep_open) device_out->batch = batch;
      else ok = cqlcuda_batch_end(batch);
      free(host_out);
      if (!ok) return 0;
      device_out->buffer = out_buf;
      device_out->sum_at = sum_at;
      device_out->min_at = min_at;
      device_out->max_at = max_at;
      device_out->group_count = group_count;
      device_out->min_key = min_key;
      return 1;
    }
    cqlcuda_batch_buffer_read(batch, out_buf, host_out, counted);
    if (!has_min_max)
    {
      for (uint64_t i = 0; i < group_count * expr_count; i++)
      {
        mins[i] = 0x7fffffffu;
        maxs[i] = 0x80000000u;
      }
    }
    ok = cqlcuda_batch_end(batch);
  }
  if (ok)
  {
    /* qe_dense_stream_retire (:7600-7628) */
    for (uint64_t g = 0; g < group_count; g++)
    {
      out_counts[g] = info[g * 2 + 1];
      for (uint32_t e = 0; e < expr_count; e++)
      {
        uint64_t i = g * expr_count + e;
        out_sums[i] = (int64_t)(((uint64_t)sums[i * 2 + 1] << 32) | (uint64_t)sums[i * 2]);
        out_mins[i] = (int64_t)(int32_t)mins[i];
        out_maxs[i] = (int64_t)(int32_t)maxs[i];
      }
    }
    *out_group_count = group_count;
    *out_min_key = min_key;
  }
  free(host_out);
  return ok;
}
