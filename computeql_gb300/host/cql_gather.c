/*
 * cql_gather.c - row materialization: the values of a selection's rows of many columns, read back to
 * host memory in selection order (selection_gather.comp modes 0/1, qe_selection_gather_column,
 * src/query_exec/query_exec.c:4371-4410, which the reference runs one column and one batch at a time).
 *
 * Here one batch uploads the selection once, gathers up to 13 columns a launch into one destination
 * buffer (each column in a 16-byte-aligned section) and reads every section straight into the caller's
 * array. Raw strings take two batches: their lengths and an exclusive scan of them (the output offsets),
 * then a warp per row copies the bytes.
 */
#include "cqlops.h"
#include "cql_ops_internal.h"

#include <stdio.h>
#include <stdlib.h>
#include <string.h>

#define GATHER_COLUMNS 13
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

/* the gather kernel's kind for a column and the bytes of one output value; 0 when it has none */
static int gather_kind(const CqlColumn* c, uint32_t* kind, uint32_t* size)
{
  if (c->width == 3)
  {
    *kind = 3;
    *size = 4;
    return c->type != CQLOPS_TYPE_F32 && c->type != CQLOPS_TYPE_BOOL;
  }
  if (c->width == 1 || c->width == 2)
  {
    *kind = c->width;
    *size = 4;
    return c->type != CQLOPS_TYPE_F32 && c->type != CQLOPS_TYPE_BOOL && c->buffer != NULL;
  }
  if (c->width != 0 || !c->buffer) return 0;
  switch (c->type)
  {
    case CQLOPS_TYPE_U32: case CQLOPS_TYPE_I32: case CQLOPS_TYPE_F32: case 9: case 12:
      *kind = 0;
      *size = 4;
      return 1;
    case CQLOPS_TYPE_U64: case CQLOPS_TYPE_I64: case CQLOPS_TYPE_F64: case 10: case 11:
      *kind = 4;
      *size = 8;
      return 1;
    case CQLOPS_TYPE_BOOL:
      *kind = 5;
      *size = 1;
      return 1;
    case CQLOPS_TYPE_STRING8:
      /* dictionary codes */
      *kind = 0;
      *size = 4;
      return c->dict != NULL;
    default:
      return 0;
  }
}

/* the selection the kernels read: the host rows uploaded into batch b, the caller's device buffer, or
   none (rows 0..count-1); 0 when a host row is past the shortest column */
static int selection_source(CqlBatch* b, const uint32_t* rows, CqlBuffer* selection, uint64_t count, uint64_t min_rows, CqlBuffer** out,
                            uint32_t* out_given)
{
  *out = NULL;
  *out_given = 0;
  if (rows)
  {
    for (uint64_t i = 0; i < count; i++)
      if (rows[i] >= min_rows) return refuse("a selected row is past the end of a column");
    CqlBuffer* up = pooled("gather_rows", count * 4, CQLCUDA_BUFFER_WRITE);
    if (!up) return 0;
    cqlcuda_batch_buffer_write(b, up, rows, count * 4);
    *out = up;
    *out_given = 1;
  }
  else if (selection)
  {
    if (cqlcuda_buffer_size(selection) < count * 4) return refuse("selection buffer smaller than its count");
    *out = selection;
    *out_given = 1;
  }
  else if (count > min_rows) return refuse("more rows asked for than the columns hold");
  return 1;
}

int cqlops_gather_rows(const CqlColumn* columns, uint32_t column_count, const uint32_t* rows, CqlBuffer* selection, uint64_t count,
                       void* const* out_values)
{
  cqlops_note_error("");
  if (column_count == 0 || count == 0) return 1;
  if (!columns || !out_values) return refuse("columns and outputs are required");
  if (!cqlops_rows_fit(count)) return 0;
  uint32_t* params = (uint32_t*)calloc((size_t)column_count * 4, sizeof(uint32_t));
  uint64_t* section = (uint64_t*)malloc((size_t)column_count * sizeof(uint64_t));
  uint32_t* sizes = (uint32_t*)malloc((size_t)column_count * sizeof(uint32_t));
  if (!params || !section || !sizes)
  {
    free(params);
    free(section);
    free(sizes);
    return refuse("out of host memory");
  }
  uint64_t min_rows = ~0ull, total = 0;
  int ok = 1;
  for (uint32_t c = 0; c < column_count && ok; c++)
  {
    uint32_t kind = 0, size = 0;
    if (!gather_kind(&columns[c], &kind, &size) || !out_values[c])
    {
      ok = refuse("gathered columns are numeric, BOOL or dictionary strings (raw strings: cqlops_gather_strings), with an output each");
      break;
    }
    if (columns[c].rows < min_rows) min_rows = columns[c].rows;
    section[c] = total;
    sizes[c] = size;
    params[c * 4 + 0] = kind;
    params[c * 4 + 1] = columns[c].base;
    params[c * 4 + 2] = (uint32_t)total;
    params[c * 4 + 3] = (uint32_t)(total >> 32);
    total += (count * size + 15) & ~15ull;
  }
  CqlBuffer* dest = ok ? pooled("gather_dest", total, CQLCUDA_BUFFER_READ_WRITE) : NULL;
  CqlBuffer* pbuf = ok ? pooled("gather_params", (uint64_t)column_count * 16, CQLCUDA_BUFFER_WRITE) : NULL;
  CqlKernel* k = ok ? cqlcuda_kernel_alloc("cql_gather_columns", strlen("cql_gather_columns")) : NULL;
  ok = ok && dest && pbuf && k;
  if (ok)
  {
    CqlBatch* b = cqlcuda_batch_begin(count * 4 + (uint64_t)column_count * 16, total);
    CqlBuffer* sel = NULL;
    uint32_t given = 0;
    ok = selection_source(b, rows, selection, count, min_rows, &sel, &given);
    if (ok)
    {
      cqlcuda_batch_buffer_write(b, pbuf, params, (uint64_t)column_count * 16);
      for (uint32_t first = 0; first < column_count; first += GATHER_COLUMNS)
      {
        uint32_t n = column_count - first < GATHER_COLUMNS ? column_count - first : GATHER_COLUMNS;
        cqlcuda_kernel_set_arg_buffer(k, 0, sel ? sel : pbuf);
        cqlcuda_kernel_set_arg_buffer_range(k, 1, pbuf, (uint64_t)first * 16, (uint64_t)n * 16);
        cqlcuda_kernel_set_arg_buffer(k, 2, dest);
        for (uint32_t j = 0; j < GATHER_COLUMNS; j++)
        {
          CqlBuffer* src = j < n ? columns[first + j].buffer : NULL;
          cqlcuda_kernel_set_arg_buffer(k, 3 + j, src ? src : pbuf);
        }
        cqlcuda_kernel_set_arg_u64(k, 0, count);
        cqlcuda_kernel_set_arg_u64(k, 1, given);
        cqlcuda_kernel_set_arg_u64(k, 2, n);
        cqlcuda_batch_kernel_execute(b, k, (uint32_t)count, QE_GPU_WORKGROUP_SIZE);
      }
      /* outputs laid out as the device sections are (one host block, each column at its section's offset):
         one read of the whole block; else a read a column */
      int contiguous = 1;
      for (uint32_t c = 1; c < column_count && contiguous; c++)
        contiguous = (const char*)out_values[c] == (const char*)out_values[0] + section[c];
      if (contiguous)
        cqlcuda_batch_buffer_read_at(b, dest, 0, out_values[0], section[column_count - 1] + count * sizes[column_count - 1]);
      else
        for (uint32_t c = 0; c < column_count; c++) cqlcuda_batch_buffer_read_at(b, dest, section[c], out_values[c], count * sizes[c]);
    }
    int ended = cqlcuda_batch_end(b);
    ok = ok && ended;
  }
  if (k) cqlcuda_kernel_release(k);
  free(params);
  free(section);
  free(sizes);
  return ok;
}

int cqlops_gather_strings(const CqlColumn* column, const uint32_t* rows, CqlBuffer* selection, uint64_t count, uint64_t* out_offsets,
                          char* out_bytes, uint64_t bytes_capacity, uint64_t* out_bytes_needed)
{
  cqlops_note_error("");
  if (out_bytes_needed) *out_bytes_needed = 0;
  if (!column || column->type != CQLOPS_TYPE_STRING8 || column->dict || !column->buffer || !column->offsets || column->width != 0)
    return refuse("cqlops_gather_strings takes a raw STRING8 column (bytes and offsets)");
  if (!out_offsets) return refuse("out_offsets must hold count + 1 offsets");
  out_offsets[0] = 0;
  if (count == 0) return 1;
  if (count >= 0xffffffffull || cqlcuda_buffer_size(column->buffer) >= 0xffffffffull) return refuse("row count or string bytes out of range");
  uint64_t blocks = (count + 255) / 256;
  CqlBuffer* lengths = pooled("gather_str_lengths", count * 4, CQLCUDA_BUFFER_READ_WRITE);
  CqlBuffer* offs = pooled("gather_str_offsets", (count + 1) * 4, CQLCUDA_BUFFER_READ_WRITE);
  CqlBuffer* cursor = pooled("gather_str_cursor", count * 4, CQLCUDA_BUFFER_READ_WRITE);
  CqlBuffer* block_sums = pooled("gather_str_block_sums", blocks * 4, CQLCUDA_BUFFER_READ_WRITE);
  CqlKernel* klen = cqlcuda_kernel_alloc("cql_gather_string_lengths", strlen("cql_gather_string_lengths"));
  CqlKernel* scan = cqlcuda_kernel_alloc("prefix_sum", strlen("prefix_sum"));
  CqlKernel* kbytes = cqlcuda_kernel_alloc("cql_gather_string_bytes", strlen("cql_gather_string_bytes"));
  uint32_t* h_off = (uint32_t*)malloc((count + 1) * 4);
  int ok = lengths && offs && cursor && block_sums && klen && scan && kbytes && h_off;
  CqlBuffer* sel = NULL;
  uint32_t given = 0;
  uint32_t total = 0;
  if (ok)
  {
    CqlBatch* b = cqlcuda_batch_begin(count * 4, 4);
    ok = selection_source(b, rows, selection, count, column->rows, &sel, &given);
    if (ok)
    {
      cqlcuda_kernel_set_arg_buffer(klen, 0, sel ? sel : lengths);
      cqlcuda_kernel_set_arg_buffer(klen, 1, column->offsets);
      cqlcuda_kernel_set_arg_buffer(klen, 2, lengths);
      cqlcuda_kernel_set_arg_u64(klen, 0, count);
      cqlcuda_kernel_set_arg_u64(klen, 1, given);
      cqlcuda_batch_kernel_execute(b, klen, (uint32_t)count, QE_GPU_WORKGROUP_SIZE);
      cqlcuda_kernel_set_arg_buffer(scan, 0, lengths);
      cqlcuda_kernel_set_arg_buffer(scan, 1, offs);
      cqlcuda_kernel_set_arg_buffer(scan, 2, cursor);
      cqlcuda_kernel_set_arg_buffer(scan, 3, block_sums);
      cqlcuda_kernel_set_arg_u64(scan, 0, count);
      for (uint32_t mode = 0; mode < 3; mode++)
      {
        cqlcuda_kernel_set_arg_u64(scan, 1, mode);
        cqlcuda_batch_kernel_execute(b, scan, mode == 1 ? 256u : (uint32_t)(blocks * 256), 256);
      }
      cqlcuda_batch_buffer_read_at(b, offs, count * 4, &total, 4);
    }
    int ended = cqlcuda_batch_end(b);
    ok = ok && ended;
  }
  if (ok)
  {
    if (out_bytes_needed) *out_bytes_needed = total;
    if (total > bytes_capacity || (total && !out_bytes)) ok = refuse("out_bytes is smaller than the selected strings (out_bytes_needed says how much they need)");
  }
  if (ok)
  {
    CqlBuffer* out = pooled("gather_str_bytes", total, CQLCUDA_BUFFER_READ_WRITE);
    ok = out != NULL;
    if (ok)
    {
      CqlBatch* b = cqlcuda_batch_begin(0, (count + 1) * 4 + total);
      cqlcuda_kernel_set_arg_buffer(kbytes, 0, sel ? sel : lengths);
      cqlcuda_kernel_set_arg_buffer(kbytes, 1, column->offsets);
      cqlcuda_kernel_set_arg_buffer(kbytes, 2, column->buffer);
      cqlcuda_kernel_set_arg_buffer(kbytes, 3, offs);
      cqlcuda_kernel_set_arg_buffer(kbytes, 4, out);
      cqlcuda_kernel_set_arg_u64(kbytes, 0, count);
      cqlcuda_kernel_set_arg_u64(kbytes, 1, given);
      cqlcuda_batch_kernel_execute(b, kbytes, (uint32_t)count, QE_GPU_WORKGROUP_SIZE);
      cqlcuda_batch_buffer_read(b, offs, h_off, (count + 1) * 4);
      if (total) cqlcuda_batch_buffer_read(b, out, out_bytes, total);
      ok = cqlcuda_batch_end(b);
    }
  }
  if (ok)
    for (uint64_t i = 0; i <= count; i++) out_offsets[i] = h_off[i];
  if (klen) cqlcuda_kernel_release(klen);
  if (scan) cqlcuda_kernel_release(scan);
  if (kbytes) cqlcuda_kernel_release(kbytes);
  free(h_off);
  return ok;
}
