/*
 * cql_ops_filter.c - WHERE filters through per-query kernels, the interpreter or scan_simple, and the
 * fused filter + aggregate / group-by operators, driven through the cqlcuda C ABI.
 *
 *  cqlops_scan_filter              qe_scan_filter_selected (src/query_exec/query_exec.c:2495-3276)
 *  cqlops_fused_filter_aggregate   qe_fused_filter_aggregate (:9888-10254)
 *  cqlops_fused_filter_group       qe_fused_filter_group_aggregate (:9442-9886)
 *
 * A generated kernel is named by two hashes of its source (qk_kernel_from_source,
 * src/query_exec/query_kernel.c:1676-1735), looked up in the backend's cache before it is compiled,
 * and a source that failed to compile is remembered and not tried again (the failed-key memo,
 * :1683-1726): the scan then runs on the interpreter.
 */
#include "cqlops.h"
#include "cql_ops_internal.h"

#include <pthread.h>
#include <stdio.h>
#include <stdlib.h>
#include <string.h>

#define QE_GPU_WORKGROUP_SIZE 256
#define QE_SCAN_MAX_STACK 8
#define FAILED_CAP 64
#define FUSE_GROUP_SHARED_WORDS 4096

const char* cqlops_last_error(void);
uint32_t cqlops_program_simple_leaves(const CqlProgram* prog, CqlLeaf* out, uint32_t cap);

/* the failed-key memo and its counters, shared by every calling thread */
static pthread_mutex_t g_failed_lock = PTHREAD_MUTEX_INITIALIZER;
static uint64_t g_failed[FAILED_CAP];
static uint32_t g_failed_count = 0;
static uint64_t g_generated_requests = 0, g_generated_failures = 0;
int cqlops_bitmap_rows(CqlBuffer* bitmap, uint64_t first_row, uint64_t rows, uint64_t count, uint32_t* out_rows, uint64_t cap);

void cqlops_generated_stats(uint64_t* out_requests, uint64_t* out_failures)
{
  pthread_mutex_lock(&g_failed_lock);
  if (out_requests) *out_requests = g_generated_requests;
  if (out_failures) *out_failures = g_generated_failures;
  pthread_mutex_unlock(&g_failed_lock);
}

/* every column the program binds fits the kernels' 32-bit row numbers */
static int program_rows_fit(const CqlProgram* prog, const CqlColumn* columns)
{
  if (!prog->binding_count) return cqlops_rows_fit(columns[0].rows);
  for (uint32_t i = 0; i < prog->binding_count; i++)
    if (!cqlops_rows_fit(columns[prog->binding_column[i]].rows)) return 0;
  return 1;
}

static int refuse(const char* why)
{
  cqlops_note_error(why);
  return 0;
}

static CqlBuffer* pooled(const char* name, uint64_t size, uint32_t flags)
{
  return cqlcuda_buffer_alloc_pooled(name, (uint64_t)strlen(name), size, flags, NULL);
}

/* two hashes of a source (qk_source_key / qk_check_hash) */
static uint64_t hash_fnv(const char* s, uint64_t n)
{
  uint64_t h = 1469598103934665603ull;
  for (uint64_t i = 0; i < n; i++)
  {
    h ^= (unsigned char)s[i];
    h *= 1099511628211ull;
  }
  return h;
}

static uint64_t hash_check(const char* s, uint64_t n)
{
  uint64_t h = 0x9e3779b97f4a7c15ull ^ n;
  for (uint64_t i = 0; i < n; i++) h = (h ^ (unsigned char)s[i]) * 0xff51afd7ed558ccdull + (h >> 29);
  return h;
}

static int failed_before(uint64_t key)
{
  int found = 0;
  pthread_mutex_lock(&g_failed_lock);
  for (uint32_t i = 0; i < g_failed_count && i < FAILED_CAP; i++)
    if (g_failed[i] == key) found = 1;
  pthread_mutex_unlock(&g_failed_lock);
  return found;
}

/* the generated kernel of `kind` for the program, from the backend's cache or NVRTC; NULL on failure */
static CqlKernel* generated_kernel(const CqlProgram* prog, uint32_t kind, const CqlFusedAgg* fuse)
{
  uint64_t len = 0;
  if (!cqlops_program_source(prog, kind, fuse, NULL, 0, &len))
  {
    char why[256];
    cqlops_program_source(prog, kind, fuse, why, sizeof(why), NULL);
    refuse(why);
    return NULL;
  }
  char* src = (char*)malloc(len + 1);
  if (!src || !cqlops_program_source(prog, kind, fuse, src, len + 1, NULL))
  {
    free(src);
    return NULL;
  }
  pthread_mutex_lock(&g_failed_lock);
  g_generated_requests += 1;
  pthread_mutex_unlock(&g_failed_lock);
  uint64_t key = hash_fnv(src, len), check = hash_check(src, len);
  char name[64];
  snprintf(name, sizeof(name), "qk_%s_%016llx%016llx", kind == CQLOPS_KERNEL_SCAN ? "scan" : (kind == CQLOPS_KERNEL_FUSED_AGG ? "fagg" : "fgrp"),
           (unsigned long long)key, (unsigned long long)check);
  if (failed_before(key ^ check))
  {
    free(src);
    refuse("this kernel's source failed to compile before");
    return NULL;
  }
  CqlKernel* k = cqlcuda_kernel_alloc_from_image(name, (uint64_t)strlen(name), src, len);
  free(src);
  if (!k)
  {
    pthread_mutex_lock(&g_failed_lock);
    g_generated_failures += 1;
    g_failed[g_failed_count++ % FAILED_CAP] = key ^ check;
    pthread_mutex_unlock(&g_failed_lock);
    refuse("the generated kernel did not compile");
  }
  return k;
}

/* binds the program's columns at 6 + slot (a raw string column also its offsets at the next slot),
   every other slot to `filler` */
static int bind_columns(CqlKernel* k, const CqlProgram* prog, const CqlColumn* columns, CqlBuffer* filler)
{
  int bound[CQLOPS_MAX_BINDINGS] = { 0 };
  for (uint32_t b = 0; b < prog->binding_count; b++)
  {
    const CqlColumn* col = &columns[prog->binding_column[b]];
    uint32_t slot = prog->binding_slot[b];
    if (!col->buffer || col->width != 0) return refuse("the per-query kernels read columns stored at full width");
    cqlcuda_kernel_set_arg_buffer(k, 6 + slot, col->buffer);
    bound[slot] = 1;
    if (col->type == CQLOPS_TYPE_STRING8 && !prog->binding_dict[b])
    {
      if (!col->offsets || slot + 1 >= CQLOPS_MAX_BINDINGS) return refuse("a string column needs its offsets");
      cqlcuda_kernel_set_arg_buffer(k, 6 + slot + 1, col->offsets);
      bound[slot + 1] = 1;
    }
  }
  for (uint32_t s = 0; s < CQLOPS_MAX_BINDINGS; s++)
    if (!bound[s]) cqlcuda_kernel_set_arg_buffer(k, 6 + s, filler);
  return 1;
}

/* the table's row count: a program that reads no column (a folded TRUE/FALSE) still runs over the
   rows of the table its columns belong to */
static uint64_t program_rows(const CqlProgram* prog, const CqlColumn* columns, uint64_t fallback)
{
  (void)fallback;
  return prog->binding_count ? columns[prog->binding_column[0]].rows : columns[0].rows;
}

/* bytecode, constants and string pool of a program into pooled buffers, written in one batch */
static int upload_program(const CqlProgram* prog, CqlBuffer** out_code, CqlBuffer** out_consts, CqlBuffer** out_strs)
{
  uint64_t code_bytes = (uint64_t)prog->word_count * 4;
  uint64_t const_bytes = (uint64_t)(prog->const_count ? prog->const_count : 1) * 8;
  uint64_t str_bytes = prog->str_pool_size ? ((prog->str_pool_size + 3u) & ~3u) : 4;
  *out_code = pooled("cqlops_scan_bytecode", code_bytes ? code_bytes : 4, CQLCUDA_BUFFER_WRITE);
  *out_consts = pooled("cqlops_scan_num_consts", const_bytes, CQLCUDA_BUFFER_WRITE);
  *out_strs = pooled("cqlops_scan_str_consts", str_bytes, CQLCUDA_BUFFER_WRITE);
  if (!*out_code || !*out_consts || !*out_strs) return 0;
  CqlBatch* batch = cqlcuda_batch_begin(code_bytes + const_bytes + str_bytes, 0);
  if (code_bytes) cqlcuda_batch_buffer_write(batch, *out_code, prog->words, code_bytes);
  if (prog->const_count) cqlcuda_batch_buffer_write(batch, *out_consts, prog->consts, (uint64_t)prog->const_count * 8);
  if (prog->str_pool_size)
  {
    uint8_t pad[CQLOPS_MAX_STR_POOL + 4];
    memset(pad, 0, str_bytes);
    memcpy(pad, prog->str_pool, prog->str_pool_size);
    cqlcuda_batch_buffer_write(batch, *out_strs, pad, str_bytes);
  }
  return cqlcuda_batch_end(batch);
}

/* scan_simple over the program's leaves, columns remapped to the leaf columns */
static int run_simple(const CqlProgram* prog, const CqlColumn* columns, const CqlLeaf* leaves, uint32_t n, uint64_t* out_count,
                      uint32_t* out_rows, uint64_t cap)
{
  CqlColumn cols[CQLOPS_MAX_BINDINGS];
  uint32_t map_from[CQLOPS_MAX_BINDINGS];
  uint32_t used = 0;
  CqlLeaf local[8];
  for (uint32_t l = 0; l < n; l++)
  {
    uint32_t c = 0;
    while (c < used && map_from[c] != leaves[l].column) c++;
    if (c == used)
    {
      if (used == CQLOPS_MAX_BINDINGS) return 0;
      map_from[used] = leaves[l].column;
      cols[used] = columns[leaves[l].column];
      used++;
    }
    local[l] = leaves[l];
    local[l].column = c;
  }
  (void)prog;
  return cqlops_scan_simple(cols, used, local, n, out_count, out_rows, cap);
}

static int scan_filter_run(const CqlProgram* prog, const CqlColumn* columns, uint32_t strategy, uint64_t* out_count, uint32_t* out_rows,
                           double* out_scores, uint64_t out_capacity, uint32_t* out_strategy)
{
  cqlops_note_error("");
  if (prog->requires_cpu_scan) return refuse("the program needs the CPU scan, which this backend does not have");
  if (!program_rows_fit(prog, columns)) return 0;
  /* a fuzzy comparison runs on the interpreter only (qe_scan_filter_selected, :2532, :2641) */
  uint32_t score_flags = prog->has_score_output ? (1u | (prog->has_score_output == 2u ? 2u : 0u)) : 0u;
  if (score_flags)
  {
    if (strategy == CQLOPS_SCAN_SIMPLE || strategy == CQLOPS_SCAN_GENERATED) return refuse("a fuzzy comparison runs on the interpreter");
    strategy = CQLOPS_SCAN_INTERPRETER;
  }
  uint64_t rows = program_rows(prog, columns, 0);
  if (rows == 0)
  {
    /* an empty table matches nothing: no device work */
    if (out_count) *out_count = 0;
    if (out_strategy) *out_strategy = strategy == CQLOPS_SCAN_AUTO ? CQLOPS_SCAN_INTERPRETER : strategy;
    return 1;
  }

  if (strategy == CQLOPS_SCAN_AUTO || strategy == CQLOPS_SCAN_SIMPLE)
  {
    CqlLeaf leaves[8];
    uint32_t n = cqlops_program_simple_leaves(prog, leaves, 8);
    if (n > 0)
    {
      if (out_strategy) *out_strategy = CQLOPS_SCAN_SIMPLE;
      return run_simple(prog, columns, leaves, n, out_count, out_rows, out_capacity);
    }
    if (strategy == CQLOPS_SCAN_SIMPLE) return refuse("the condition is not an AND of numeric comparisons");
  }

  CqlKernel* k = NULL;
  uint32_t ran = strategy == CQLOPS_SCAN_INTERPRETER ? CQLOPS_SCAN_INTERPRETER : CQLOPS_SCAN_GENERATED;
  if (ran == CQLOPS_SCAN_GENERATED)
  {
    k = generated_kernel(prog, CQLOPS_KERNEL_SCAN, NULL);
    if (!k && strategy == CQLOPS_SCAN_GENERATED) return 0;
    if (!k) ran = CQLOPS_SCAN_INTERPRETER;
  }
  if (ran == CQLOPS_SCAN_INTERPRETER)
  {
    if (cqlops_program_max_stack_depth(prog) > QE_SCAN_MAX_STACK) return refuse("the program is deeper than the interpreter's stack");
    k = cqlcuda_kernel_alloc("scan_filter", 11);
    if (!k) return 0;
  }
  CqlBuffer *code, *consts, *strs;
  if (!upload_program(prog, &code, &consts, &strs)) return 0;
  CqlBuffer* counter = pooled("scan_filter_result_counter", 8, CQLCUDA_BUFFER_READ_WRITE);
  CqlBuffer* filler = pooled("cqlops_filler", 16, CQLCUDA_BUFFER_WRITE);
  if (!counter || !filler) return 0;
  if (!bind_columns(k, prog, columns, filler)) return 0;
  cqlcuda_kernel_set_arg_buffer(k, 0, code);
  cqlcuda_kernel_set_arg_buffer(k, 1, consts);
  cqlcuda_kernel_set_arg_buffer(k, 2, strs);
  cqlcuda_kernel_set_arg_buffer(k, 4, counter);
  cqlcuda_kernel_set_arg_buffer(k, 5, filler);
  cqlcuda_kernel_set_arg_u64(k, 0, rows);
  cqlcuda_kernel_set_arg_u64(k, 1, score_flags);   /* word 2: bit 0 score output, bit 1 a distance */
  cqlcuda_kernel_set_arg_u64(k, 2, 3);             /* word 4: the trigram length */
  cqlcuda_kernel_set_arg_u64(k, 3, 0);
  cqlcuda_kernel_set_arg_u64(k, 4, 0);

  int want_rows = out_rows != NULL || out_scores != NULL;
  /* rows without scores: the kernel writes a bitmap of the rows (word 10), which becomes ascending rows
     on the device; no output capacity, no second run, no host sort */
  int bitmap = want_rows && !score_flags && out_scores == NULL;
  cqlcuda_kernel_set_arg_u64(k, 5, bitmap ? 1 : 0);
  if (bitmap)
  {
    uint64_t words = (rows + 31) / 32;
    CqlBuffer* bits = pooled("scan_bitmap", words * 4, CQLCUDA_BUFFER_READ_WRITE);
    if (!bits) return 0;
    cqlcuda_kernel_set_arg_buffer(k, 3, bits);
    uint32_t c32[2] = { 0, 0 };
    CqlBatch* batch = cqlcuda_batch_begin(0, 8);
    cqlcuda_batch_buffer_zero(batch, counter, 8);
    cqlcuda_batch_kernel_execute(batch, k, (uint32_t)(rows < 0xffffffffull ? rows : 0xffffffffull), QE_GPU_WORKGROUP_SIZE);
    cqlcuda_batch_buffer_read(batch, counter, c32, 8);
    if (!cqlcuda_batch_end(batch)) return 0;
    if (!cqlops_bitmap_rows(bits, 0, rows, c32[0], out_rows, out_capacity)) return 0;
    if (out_count) *out_count = c32[0];
    if (out_strategy) *out_strategy = ran;
    return 1;
  }
  uint64_t cap_rows = 0;
  if (want_rows)
  {
    uint64_t d = rows / 32 > 65536 ? rows / 32 : 65536;
    cap_rows = d < rows ? d : rows;
    if (!cap_rows) cap_rows = 1;
  }
  uint64_t result = 0;
  CqlBuffer* output = NULL;
  for (int attempt = 0; attempt < 2; attempt++)
  {
    output = want_rows ? pooled("scan_filter_output", cap_rows * 8, CQLCUDA_BUFFER_READ) : pooled("cqlops_scan_no_output", 0, CQLCUDA_BUFFER_READ);
    if (!output) return 0;
    cqlcuda_kernel_set_arg_buffer(k, 3, output);
    uint32_t c32[2] = { 0, 0 };
    CqlBatch* batch = cqlcuda_batch_begin(0, 8);
    cqlcuda_batch_buffer_zero(batch, counter, 8);
    cqlcuda_batch_kernel_execute(batch, k, (uint32_t)(rows < 0xffffffffull ? rows : 0xffffffffull), QE_GPU_WORKGROUP_SIZE);
    cqlcuda_batch_buffer_read(batch, counter, c32, 8);
    if (!cqlcuda_batch_end(batch)) return 0;
    result = c32[0];
    if (!want_rows || result <= cap_rows) break;
    cap_rows = result;
  }
  if (want_rows && result > cap_rows) return 0;
  if (want_rows && result && out_capacity)
  {
    /* the kernel's order is not deterministic: (row, score) pairs sorted by row on the device */
    uint64_t m = result < out_capacity ? result : out_capacity;
    uint32_t* pairs = (uint32_t*)malloc(m * 8);
    if (!pairs) return 0;
    if (!cqlops_sort_pairs(output, result, 2, 0, 1, 0, pairs, out_capacity))
    {
      free(pairs);
      return 0;
    }
    for (uint64_t i = 0; i < m; i++)
    {
      if (out_rows) out_rows[i] = pairs[2 * i];
      if (out_scores)
      {
        uint32_t aux = pairs[2 * i + 1];
        float f;
        memcpy(&f, &aux, 4);
        out_scores[i] = !score_flags ? 0.0 : (score_flags & 2u) ? (double)aux : (double)f;
      }
    }
    free(pairs);
  }
  if (out_count) *out_count = result;
  if (out_strategy) *out_strategy = ran;
  return 1;
}

int cqlops_scan_filter(const CqlProgram* prog, const CqlColumn* columns, uint32_t strategy, uint64_t* out_count, uint32_t* out_rows,
                       uint64_t out_capacity, uint32_t* out_strategy)
{
  return scan_filter_run(prog, columns, strategy, out_count, out_rows, NULL, out_capacity, out_strategy);
}

int cqlops_scan_filter_scored(const CqlProgram* prog, const CqlColumn* columns, uint64_t* out_count, uint32_t* out_rows, double* out_scores,
                              uint64_t out_capacity)
{
  return scan_filter_run(prog, columns, CQLOPS_SCAN_AUTO, out_count, out_rows, out_scores, out_capacity, NULL);
}

int cqlops_fused_filter_aggregate(const CqlProgram* prog_in, const CqlColumn* columns, const uint32_t* agg_columns, uint32_t agg_count,
                                  double* out_count, double* out_sum, double* out_min, double* out_max)
{
  cqlops_note_error("");
  if (agg_count > 4) return refuse("at most 4 aggregate columns");
  if (prog_in->requires_cpu_scan || prog_in->has_score_output) return refuse("the program needs the CPU scan");
  if (!program_rows_fit(prog_in, columns)) return 0;
  CqlProgram* prog = (CqlProgram*)malloc(sizeof(CqlProgram));
  if (!prog) return 0;
  memcpy(prog, prog_in, sizeof(CqlProgram));
  CqlFusedAgg fuse;
  memset(&fuse, 0, sizeof(fuse));
  fuse.column_count = agg_count;
  int ok = 1;
  for (uint32_t c = 0; c < agg_count && ok; c++)
  {
    const CqlColumn* col = &columns[agg_columns[c]];
    if (!(col->type == CQLOPS_TYPE_U32 || col->type == CQLOPS_TYPE_I32 || col->type == CQLOPS_TYPE_F32 || col->type == CQLOPS_TYPE_F64 ||
          col->type == CQLOPS_TYPE_U64 || col->type == CQLOPS_TYPE_I64))
      ok = refuse("aggregate columns must be numeric");
    int slot = ok ? cqlops_program_bind(prog, columns, agg_columns[c]) : -1;
    if (slot < 0) ok = 0;
    else
    {
      fuse.slots[c] = (uint32_t)slot;
      fuse.coltypes[c] = col->type;
    }
  }

  if (ok && program_rows(prog, columns, 0) == 0)
  {
    /* an empty table: no matched rows, sums 0 and the fold's starting extremes (no device work) */
    if (out_count) *out_count = 0.0;
    for (uint32_t c = 0; c < agg_count; c++)
    {
      if (out_sum) out_sum[c] = 0.0;
      if (out_min) out_min[c] = 1.7976931348623157e308;
      if (out_max) out_max[c] = -1.7976931348623157e308;
    }
    free(prog);
    return 1;
  }
  CqlKernel* k = ok ? generated_kernel(prog, CQLOPS_KERNEL_FUSED_AGG, &fuse) : NULL;
  CqlBuffer *code = NULL, *consts = NULL, *strs = NULL;
  if (k) ok = upload_program(prog, &code, &consts, &strs);
  else ok = 0;
  uint64_t rows = ok ? program_rows(prog, columns, 0) : 0;
  uint64_t groups = rows / 65536;
  if (groups > 2048) groups = 2048;
  if (groups < 1) groups = 1;
  uint64_t width = 1 + 3 * (uint64_t)agg_count;
  CqlBuffer* partials_buf = ok ? pooled("fused_agg_partials", groups * width * 8, CQLCUDA_BUFFER_READ_WRITE) : NULL;
  CqlBuffer* filler = ok ? pooled("cqlops_filler", 16, CQLCUDA_BUFFER_WRITE) : NULL;
  double* partials = ok ? (double*)malloc(groups * width * 8) : NULL;
  if (ok && (!partials_buf || !filler || !partials)) ok = 0;
  if (ok) ok = bind_columns(k, prog, columns, filler);
  if (ok)
  {
    cqlcuda_kernel_set_arg_buffer(k, 0, filler);
    cqlcuda_kernel_set_arg_buffer(k, 1, consts);
    cqlcuda_kernel_set_arg_buffer(k, 2, strs);
    cqlcuda_kernel_set_arg_buffer(k, 3, partials_buf);
    cqlcuda_kernel_set_arg_buffer(k, 4, filler);
    cqlcuda_kernel_set_arg_buffer(k, 5, filler);
    cqlcuda_kernel_set_arg_u64(k, 0, rows);
    cqlcuda_kernel_set_arg_u64(k, 1, 0);
    cqlcuda_kernel_set_arg_u64(k, 2, 3);
    cqlcuda_kernel_set_arg_u64(k, 3, 0);
    cqlcuda_kernel_set_arg_u64(k, 4, 0);
    cqlcuda_kernel_set_arg_u64(k, 6, groups);
    CqlBatch* batch = cqlcuda_batch_begin(0, groups * width * 8);
    cqlcuda_batch_kernel_execute(batch, k, (uint32_t)(groups * QE_GPU_WORKGROUP_SIZE), QE_GPU_WORKGROUP_SIZE);
    cqlcuda_batch_buffer_read(batch, partials_buf, partials, groups * width * 8);
    ok = cqlcuda_batch_end(batch);
  }
  if (ok)
  {
    /* combined in workgroup order (:10200-10219) */
    double matched = 0.0;
    double sum[4] = { 0, 0, 0, 0 }, mn[4], mx[4];
    for (uint32_t c = 0; c < 4; c++)
    {
      mn[c] = 1.7976931348623157e308;
      mx[c] = -1.7976931348623157e308;
    }
    for (uint64_t g = 0; g < groups; g++)
    {
      const double* row = &partials[g * width];
      matched += row[0];
      for (uint32_t c = 0; c < agg_count; c++)
      {
        sum[c] += row[1 + 3 * c];
        mn[c] = row[2 + 3 * c] < mn[c] ? row[2 + 3 * c] : mn[c];
        mx[c] = row[3 + 3 * c] > mx[c] ? row[3 + 3 * c] : mx[c];
      }
    }
    if (out_count) *out_count = matched;
    for (uint32_t c = 0; c < agg_count; c++)
    {
      if (out_sum) out_sum[c] = sum[c];
      if (out_min) out_min[c] = mn[c];
      if (out_max) out_max[c] = mx[c];
    }
  }
  free(partials);
  free(prog);
  return ok;
}

int cqlops_fused_filter_group(const CqlProgram* prog_in, const CqlColumn* columns, const uint32_t* key_columns, uint32_t key_count,
                              const uint32_t* agg_columns, uint32_t agg_count, uint64_t max_groups, uint64_t* out_group_total,
                              int64_t* out_key_min, uint32_t* out_key_range, uint64_t* out_counts, uint64_t* out_min_row, int64_t* out_sums,
                              int64_t* out_mins, int64_t* out_maxs)
{
  cqlops_note_error("");
  if (key_count == 0 || key_count > 3 || agg_count > 4) return refuse("1 to 3 keys and at most 4 aggregate columns");
  if (prog_in->requires_cpu_scan || prog_in->has_score_output) return refuse("the program needs the CPU scan");
  if (!program_rows_fit(prog_in, columns)) return 0;
  if (columns[key_columns[0]].rows == 0)
  {
    /* an empty table has no groups (no device work) */
    if (out_group_total) *out_group_total = 0;
    for (uint32_t k = 0; k < key_count; k++)
    {
      if (out_key_min) out_key_min[k] = 0;
      if (out_key_range) out_key_range[k] = 0;
    }
    return 1;
  }
  CqlProgram* prog = (CqlProgram*)malloc(sizeof(CqlProgram));
  if (!prog) return 0;
  memcpy(prog, prog_in, sizeof(CqlProgram));
  CqlFusedAgg fuse;
  memset(&fuse, 0, sizeof(fuse));
  fuse.grouped = 1;
  fuse.key_count = key_count;
  fuse.column_count = agg_count;
  int32_t key_min[3] = { 0, 0, 0 };
  uint64_t total = 1;
  int ok = 1;
  /* the keys: whole-number columns with a small zone range, or dictionary codes (:9466-9521) */
  for (uint32_t k = 0; k < key_count && ok; k++)
  {
    const CqlColumn* col = &columns[key_columns[k]];
    uint64_t range;
    if (col->type == CQLOPS_TYPE_STRING8)
    {
      if (!col->dict) ok = refuse("a string key needs its dictionary");
      key_min[k] = 0;
      range = ok ? col->dict->count : 0;
    }
    else
    {
      if ((col->type != CQLOPS_TYPE_U32 && col->type != CQLOPS_TYPE_I32) || !col->has_range || col->zone_min < -2147483648.0 ||
          col->zone_max > 2147483647.0)
        ok = refuse("keys must be U32/I32 columns with a zone range");
      key_min[k] = (int32_t)col->zone_min;
      range = ok ? (uint64_t)(col->zone_max - col->zone_min) + 1 : 0;
    }
    total *= range;
    if (ok && (range == 0 || total > 0xffffffffull)) ok = refuse("too many groups");
    if (!ok) break;
    int slot = cqlops_program_bind(prog, columns, key_columns[k]);
    if (slot < 0)
    {
      ok = 0;
      break;
    }
    uint32_t b = 0;
    while (b < prog->binding_count && prog->binding_slot[b] != (uint32_t)slot) b++;
    fuse.key_slots[k] = (uint32_t)slot;
    fuse.key_types[k] = prog->binding_type[b];
    fuse.key_ranges[k] = (uint32_t)range;
  }
  for (uint32_t c = 0; c < agg_count && ok; c++)
  {
    const CqlColumn* col = &columns[agg_columns[c]];
    if (col->type != CQLOPS_TYPE_U32 && col->type != CQLOPS_TYPE_I32) ok = refuse("sums are exact only for U32/I32 arguments");
    int slot = ok ? cqlops_program_bind(prog, columns, agg_columns[c]) : -1;
    if (slot < 0) ok = 0;
    else
    {
      fuse.slots[c] = (uint32_t)slot;
      fuse.coltypes[c] = col->type;
    }
  }
  uint32_t width = 2 + 4 * agg_count;
  if (ok && total * width > FUSE_GROUP_SHARED_WORDS) ok = refuse("the groups do not fit the fused kernel's 16 KB table");
  if (ok && total > max_groups) ok = refuse("the output arrays are too small for the groups");
  fuse.group_count = (uint32_t)total;
  CqlKernel* kern = ok ? generated_kernel(prog, CQLOPS_KERNEL_FUSED_GROUP, &fuse) : NULL;
  CqlBuffer *code = NULL, *consts = NULL, *strs = NULL;
  ok = kern && upload_program(prog, &code, &consts, &strs);
  uint64_t rows = ok ? program_rows(prog, columns, 0) : 0;
  uint64_t words = total * width;
  CqlBuffer* out_buf = ok ? pooled("fused_group_output", words * 4, CQLCUDA_BUFFER_READ_WRITE) : NULL;
  CqlBuffer* filler = ok ? pooled("cqlops_filler", 16, CQLCUDA_BUFFER_WRITE) : NULL;
  uint32_t* init = ok ? (uint32_t*)calloc(words, 4) : NULL;
  uint32_t* result = ok ? (uint32_t*)malloc(words * 4) : NULL;
  if (ok && (!out_buf || !filler || !init || !result)) ok = 0;
  if (ok) ok = bind_columns(kern, prog, columns, filler);
  if (ok)
  {
    /* the identity of every merge: counts and sums 0, smallest row and minimums all ones (:9701-9711) */
    for (uint64_t g = 0; g < total; g++)
    {
      init[g * width + 1] = 0xffffffffu;
      for (uint32_t c = 0; c < agg_count; c++) init[g * width + 4 + 4 * c] = 0xffffffffu;
    }
    uint64_t wgs = rows / 131072;
    if (wgs > 1024) wgs = 1024;
    if (wgs < 1) wgs = 1;
    cqlcuda_kernel_set_arg_buffer(kern, 0, filler);
    cqlcuda_kernel_set_arg_buffer(kern, 1, consts);
    cqlcuda_kernel_set_arg_buffer(kern, 2, strs);
    cqlcuda_kernel_set_arg_buffer(kern, 3, out_buf);
    cqlcuda_kernel_set_arg_buffer(kern, 4, filler);
    cqlcuda_kernel_set_arg_buffer(kern, 5, filler);
    cqlcuda_kernel_set_arg_u64(kern, 0, rows);
    cqlcuda_kernel_set_arg_u64(kern, 1, 0);
    cqlcuda_kernel_set_arg_u64(kern, 2, 3);
    cqlcuda_kernel_set_arg_u64(kern, 3, 0);
    cqlcuda_kernel_set_arg_u64(kern, 4, 0);
    cqlcuda_kernel_set_arg_u64(kern, 6, wgs | ((uint64_t)(uint32_t)key_min[2] << 32));
    cqlcuda_kernel_set_arg_u64(kern, 7, (uint64_t)(uint32_t)key_min[0] | ((uint64_t)(uint32_t)key_min[1] << 32));
    CqlBatch* batch = cqlcuda_batch_begin(words * 4, words * 4);
    cqlcuda_batch_buffer_write(batch, out_buf, init, words * 4);
    cqlcuda_batch_kernel_execute(batch, kern, (uint32_t)(wgs * QE_GPU_WORKGROUP_SIZE), QE_GPU_WORKGROUP_SIZE);
    cqlcuda_batch_buffer_read(batch, out_buf, result, words * 4);
    ok = cqlcuda_batch_end(batch);
  }
  if (ok)
  {
    /* decode (:9817-9860): an I32 argument was summed and compared with its sign bit flipped */
    for (uint64_t g = 0; g < total; g++)
    {
      const uint32_t* grp = &result[g * width];
      out_counts[g] = grp[0];
      out_min_row[g] = grp[0] ? grp[1] : UINT64_MAX;
      for (uint32_t c = 0; c < agg_count; c++)
      {
        int is_signed = columns[agg_columns[c]].type == CQLOPS_TYPE_I32;
        uint64_t sum_bits = ((uint64_t)grp[3 + 4 * c] << 32) | grp[2 + 4 * c];
        out_sums[g * agg_count + c] = (int64_t)sum_bits - (is_signed ? (int64_t)grp[0] * 2147483648ll : 0);
        uint32_t lo = grp[4 + 4 * c], hi = grp[5 + 4 * c];
        out_mins[g * agg_count + c] = is_signed ? (int64_t)(int32_t)(lo ^ 0x80000000u) : (int64_t)lo;
        out_maxs[g * agg_count + c] = is_signed ? (int64_t)(int32_t)(hi ^ 0x80000000u) : (int64_t)hi;
      }
    }
    *out_group_total = total;
    for (uint32_t k = 0; k < key_count; k++)
    {
      if (out_key_min) out_key_min[k] = key_min[k];
      if (out_key_range) out_key_range[k] = fuse.key_ranges[k];
    }
  }
  free(init);
  free(result);
  free(prog);
  return ok;
}
