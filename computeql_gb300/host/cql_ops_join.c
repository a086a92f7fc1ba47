/*
 * cql_ops_join.c - hash joins and the join-aggregate pushdown, driven through the cqlcuda C ABI.
 *
 *  cqlops_hash_join       qe_hash_join_impl (src/query_exec/query_exec.c:14541-15358): build-side bucket
 *                         histogram, three-pass prefix sum, scatter into bucket lists, probe emitting
 *                         (probe row, build row) pairs, LEFT JOIN unmatched rows, output capacity
 *                         max(probe, build) + probe (qe_join_output_capacity :14368-14381) grown once
 *  cqlops_join_aggregate  qe_aggregate_join_pushdown (:8442-8776): the fact table reduced to totals per
 *                         join key - densely when the fact key's range is small (qe_dense_stream_core),
 *                         else by probing a CPU-built linear-probing table of the dim keys behind a Bloom
 *                         filter (qe_join_probe_stream_core :8080-8420) - then every (filtered) dim row
 *                         meets its key's totals and is folded into a group of its group columns on the host
 */
#include "cqlops.h"
#include "cql_ops_internal.h"
#include "cql_pool.h"

#include <math.h>
#include <stdio.h>
#include <stdlib.h>
#include <string.h>

#define QE_GPU_WORKGROUP_SIZE 256
#define PROBE_STREAM_MAX_DIM_ROWS (1ull << 26)

static int refuse(const char* why)
{
  cqlops_note_error(why);
  return 0;
}

static CqlBuffer* pooled(const char* name, uint64_t size, uint32_t flags)
{
  return cqlcuda_buffer_alloc_pooled(name, (uint64_t)strlen(name), size ? size : 4, flags, NULL);
}

static CqlKernel* kernel(const char* name)
{
  return cqlcuda_kernel_alloc(name, (uint64_t)strlen(name));
}

/* a join key as the join kernels read it: f64 values (widened on the device) or raw strings */
static int join_key(const CqlColumn* col, const char* name, CqlBuffer** data, CqlBuffer** off, int* is_str)
{
  if (col->type == CQLOPS_TYPE_STRING8)
  {
    if (!col->offsets || col->dict) return refuse("a string join key is read as raw bytes and offsets");
    *data = col->buffer;
    *off = col->offsets;
    *is_str = 1;
    return 1;
  }
  if (col->width != 0 || !col->buffer) return refuse("a join key must be stored at full width");
  CqlBuffer* out = pooled(name, col->rows * 8, CQLCUDA_BUFFER_READ_WRITE);
  CqlKernel* k = kernel("cql_widen_f64");
  if (!out || !k) return 0;
  cqlcuda_kernel_set_arg_buffer(k, 0, col->buffer);
  cqlcuda_kernel_set_arg_buffer(k, 1, out);
  cqlcuda_kernel_set_arg_u64(k, 0, col->rows);
  cqlcuda_kernel_set_arg_u64(k, 1, col->type);
  CqlBatch* b = cqlcuda_batch_begin(0, 0);
  cqlcuda_batch_kernel_execute(b, k, (uint32_t)col->rows, QE_GPU_WORKGROUP_SIZE);
  if (!cqlcuda_batch_end(b)) return 0;
  *data = out;
  *off = out;
  *is_str = 0;
  return 1;
}

int cqlops_hash_join(const CqlColumn* build_key, const CqlColumn* probe_key, int left_join, uint64_t hint_pairs, uint64_t* out_count,
                     uint32_t* out_pairs, uint64_t out_capacity)
{
  cqlops_note_error("");
  uint64_t brows = build_key->rows, prows = probe_key->rows;
  if (!cqlops_rows_fit(brows) || !cqlops_rows_fit(prows)) return 0;
  if (prows == 0 || brows == 0)
  {
    /* an empty side, no device work: no pairs, or under LEFT every probe row unmatched (build row EMPTY) */
    uint64_t produced = (brows == 0 && left_join) ? prows : 0;
    for (uint64_t r = 0; out_pairs && r < produced && r < out_capacity; r++)
    {
      out_pairs[2 * r] = (uint32_t)r;
      out_pairs[2 * r + 1] = 0xffffffffu;
    }
    *out_count = produced;
    return 1;
  }
  CqlBuffer *bd, *bo, *pd, *po;
  int bstr, pstr;
  if (!join_key(build_key, "hj_build_f64", &bd, &bo, &bstr) || !join_key(probe_key, "hj_probe_f64", &pd, &po, &pstr)) return 0;
  if (bstr != pstr) return refuse("the two join keys must both be strings or both numeric");
  uint64_t buckets = 1;
  while (buckets < brows) buckets <<= 1;
  uint64_t blocks = (buckets + 255) / 256;
  CqlBuffer* counts = pooled("hj_bucket_count_buf", buckets * 4, CQLCUDA_BUFFER_READ_WRITE);
  CqlBuffer* row_bucket = pooled("hj_row_bucket_buf", (brows ? brows : 1) * 4, CQLCUDA_BUFFER_READ_WRITE);
  CqlBuffer* offsets = pooled("hj_bucket_offsets_buf", (buckets + 1) * 4, CQLCUDA_BUFFER_READ_WRITE);
  CqlBuffer* cursor = pooled("hj_cursor_buf", buckets * 4, CQLCUDA_BUFFER_READ_WRITE);
  CqlBuffer* block_sums = pooled("hj_block_sum_buf", blocks * 4, CQLCUDA_BUFFER_READ_WRITE);
  CqlBuffer* bucket_rows = pooled("hj_bucket_rows_buf", (brows ? brows : 1) * 4, CQLCUDA_BUFFER_READ_WRITE);
  CqlBuffer* pair_count = pooled("hj_out_count_buf", 4, CQLCUDA_BUFFER_READ_WRITE);
  CqlKernel* build = kernel("hash_join_build_count");
  CqlKernel* scan = kernel("prefix_sum");
  CqlKernel* scatter = kernel("csr_scatter");
  CqlKernel* probe = kernel("hash_join_probe");
  if (!counts || !row_bucket || !offsets || !cursor || !block_sums || !bucket_rows || !pair_count || !build || !scan || !scatter || !probe) return 0;
  cqlcuda_kernel_set_arg_buffer(build, 0, bd);
  cqlcuda_kernel_set_arg_buffer(build, 1, bo);
  cqlcuda_kernel_set_arg_buffer(build, 2, counts);
  cqlcuda_kernel_set_arg_buffer(build, 3, row_bucket);
  cqlcuda_kernel_set_arg_u64(build, 0, brows);
  cqlcuda_kernel_set_arg_u64(build, 1, buckets);
  cqlcuda_kernel_set_arg_u64(build, 2, (uint64_t)bstr);
  cqlcuda_kernel_set_arg_buffer(scan, 0, counts);
  cqlcuda_kernel_set_arg_buffer(scan, 1, offsets);
  cqlcuda_kernel_set_arg_buffer(scan, 2, cursor);
  cqlcuda_kernel_set_arg_buffer(scan, 3, block_sums);
  cqlcuda_kernel_set_arg_u64(scan, 0, buckets);
  cqlcuda_kernel_set_arg_buffer(scatter, 0, row_bucket);
  cqlcuda_kernel_set_arg_buffer(scatter, 1, cursor);
  cqlcuda_kernel_set_arg_buffer(scatter, 2, bucket_rows);
  cqlcuda_kernel_set_arg_u64(scatter, 0, brows);
  cqlcuda_kernel_set_arg_u64(scatter, 1, 0);   /* build keys may repeat: combine a warp's rows of one bucket */
  {
    CqlBatch* b = cqlcuda_batch_begin(0, 0);
    cqlcuda_batch_buffer_zero(b, counts, buckets * 4);
    cqlcuda_batch_kernel_execute(b, build, (uint32_t)brows, QE_GPU_WORKGROUP_SIZE);
    for (uint32_t mode = 0; mode < 3; mode++)
    {
      cqlcuda_kernel_set_arg_u64(scan, 1, mode);
      cqlcuda_batch_kernel_execute(b, scan, mode == 1 ? 256u : (uint32_t)(blocks * 256), 256);
    }
    cqlcuda_batch_kernel_execute(b, scatter, (uint32_t)brows, QE_GPU_WORKGROUP_SIZE);
    if (!cqlcuda_batch_end(b)) return 0;
  }
  uint64_t capacity = (prows > brows ? prows : brows) + prows;
  if (hint_pairs > 0)
  {
    uint64_t hinted = hint_pairs + hint_pairs / 4 + 16;
    if (hinted > capacity) capacity = hinted;
  }
  if (capacity > 0xffffffffull) capacity = 0xffffffffull;
  if (capacity < 1) capacity = 1;
  uint32_t produced = 0;
  CqlBuffer* pairs = NULL;
  for (int attempt = 0; attempt < 2; attempt++)
  {
    pairs = pooled("hj_out_pairs_buf", capacity * 16, CQLCUDA_BUFFER_READ_WRITE);
    if (!pairs) return 0;
    cqlcuda_kernel_set_arg_buffer(probe, 0, bd);
    cqlcuda_kernel_set_arg_buffer(probe, 1, bo);
    cqlcuda_kernel_set_arg_buffer(probe, 2, offsets);
    cqlcuda_kernel_set_arg_buffer(probe, 3, bucket_rows);
    cqlcuda_kernel_set_arg_buffer(probe, 4, pd);
    cqlcuda_kernel_set_arg_buffer(probe, 5, po);
    cqlcuda_kernel_set_arg_buffer(probe, 6, pairs);
    cqlcuda_kernel_set_arg_buffer(probe, 7, pair_count);
    cqlcuda_kernel_set_arg_u64(probe, 0, prows);
    cqlcuda_kernel_set_arg_u64(probe, 1, buckets);
    cqlcuda_kernel_set_arg_u64(probe, 2, (uint64_t)(left_join != 0));
    cqlcuda_kernel_set_arg_u64(probe, 3, (uint64_t)pstr);
    cqlcuda_kernel_set_arg_u64(probe, 4, capacity);
    CqlBatch* b = cqlcuda_batch_begin(0, 4);
    cqlcuda_batch_buffer_zero(b, pair_count, 4);
    cqlcuda_batch_kernel_execute(b, probe, (uint32_t)prows, QE_GPU_WORKGROUP_SIZE);
    cqlcuda_batch_buffer_read(b, pair_count, &produced, 4);
    if (!cqlcuda_batch_end(b)) return 0;
    if (produced <= capacity) break;
    capacity = produced;
  }
  if (produced > capacity) return refuse("the join produced more pairs than its output could hold");
  /* (probe row, build row) ascending, sorted on the device: words 0 and 2 of each 16-byte record */
  if (out_pairs && produced && !cqlops_sort_pairs(pairs, produced, 4, 0, 2, 1, out_pairs, out_capacity)) return 0;
  *out_count = produced;
  return 1;
}

int cqlops_group_dense(const CqlColumn* key, uint64_t rows, uint32_t expr_count, const uint32_t* funcs, const CqlColumn* const* arg_cols,
                       uint64_t max_groups, uint64_t* out_group_count, int64_t* out_min_key, uint64_t* out_counts, int64_t* out_sums,
                       int64_t* out_mins, int64_t* out_maxs);

/* totals per dim row by probing a table of the dim keys (qe_join_probe_stream_core) */
static int probe_totals(const CqlJoinAgg* q, uint32_t core_count, const uint32_t* core_funcs, const CqlColumn* const* core_cols,
                        uint64_t* counts, int64_t* sums, int64_t* mins, int64_t* maxs)
{
  const CqlColumn* fk = q->fact_key;
  uint64_t rows = fk->rows;
  uint64_t table_rows = q->dim_rows ? q->dim_count : q->dim_table_rows;
  if (q->dim_table_rows == 0 || q->dim_table_rows > PROBE_STREAM_MAX_DIM_ROWS) return refuse("dim table size out of range");
  const CqlColumn* arg_columns[4] = { 0 };
  uint32_t arg_count = 0, func_codes = 0, arg_index_codes = 0, arg_signed_bits = 0;
  for (uint32_t e = 0; e < core_count; e++)
  {
    func_codes |= (core_funcs[e] & 0xfu) << (4 * e);
    if (core_funcs[e] == CQLOPS_FUNC_COUNT) continue;
    const CqlColumn* c = core_cols[e];
    if (!c || !(c->type == CQLOPS_TYPE_U32 || c->type == CQLOPS_TYPE_I32) || c->rows != rows || c->width == 3)
      return refuse("probe aggregates take U32/I32 fact columns");
    if ((core_funcs[e] == CQLOPS_FUNC_MIN || core_funcs[e] == CQLOPS_FUNC_MAX) &&
        (!c->has_range || c->zone_min < -2147483648.0 || c->zone_max > 2147483647.0))
      return refuse("MIN/MAX values must fit a signed 32-bit word");
    uint32_t idx = 0;
    while (idx < arg_count && arg_columns[idx] != c) idx++;
    if (idx == arg_count)
    {
      if (arg_count == 4) return refuse("at most 4 argument columns");
      arg_columns[arg_count++] = c;
    }
    arg_index_codes |= (idx & 0xfu) << (4 * e);
    if (c->type == CQLOPS_TYPE_I32) arg_signed_bits |= 1u << idx;
  }
  /* the table: twice the keys, a power of two; a duplicate dim key refuses, as the reference does */
  uint32_t log2_size = 4;
  while ((1ull << log2_size) < table_rows * 2) log2_size++;
  uint64_t size = 1ull << log2_size;
  uint32_t* tkeys = (uint32_t*)calloc(size, 4);
  uint32_t* trows = (uint32_t*)calloc(size, 4);
  uint32_t bloom_log2 = 4;
  while ((1ull << bloom_log2) * 2 < table_rows) bloom_log2++;
  uint32_t* bloom = (uint32_t*)calloc(1ull << bloom_log2, 4);
  int ok = tkeys && trows && bloom;
  for (uint64_t v = 0; ok && v < table_rows; v++)
  {
    uint64_t dim_row = q->dim_rows ? q->dim_rows[v] : v;
    uint32_t key = q->dim_keys[dim_row];
    uint64_t slot = (uint32_t)(key * 0x9E3779B1u) >> (32 - log2_size);
    while (trows[slot] != 0)
    {
      if (tkeys[slot] == key)
      {
        ok = refuse("a dim key appears twice");
        break;
      }
      slot = (slot + 1) & (size - 1);
    }
    if (!ok) break;
    tkeys[slot] = key;
    trows[slot] = (uint32_t)dim_row + 1;
    uint32_t h = key * 0x9E3779B1u, h2 = key * 0x85EBCA6Bu;
    bloom[h >> (32 - bloom_log2)] |= (1u << ((h2 >> 27) & 31)) | (1u << ((h2 >> 22) & 31));
  }
  uint64_t D = q->dim_table_rows;
  CqlBuffer* kb = ok ? pooled("jp_table_keys", size * 4, CQLCUDA_BUFFER_WRITE) : NULL;
  CqlBuffer* rb = ok ? pooled("jp_table_rows", size * 4, CQLCUDA_BUFFER_WRITE) : NULL;
  CqlBuffer* bb = ok ? pooled("jp_bloom", (1ull << bloom_log2) * 4, CQLCUDA_BUFFER_WRITE) : NULL;
  CqlBuffer* cb = ok ? pooled("jp_counts", D * 4, CQLCUDA_BUFFER_READ_WRITE) : NULL;
  CqlBuffer* sb = ok ? pooled("jp_sums", D * core_count * 8, CQLCUDA_BUFFER_READ_WRITE) : NULL;
  CqlBuffer* nb = ok ? pooled("jp_mins", D * core_count * 4, CQLCUDA_BUFFER_READ_WRITE) : NULL;
  CqlBuffer* xb = ok ? pooled("jp_maxs", D * core_count * 4, CQLCUDA_BUFFER_READ_WRITE) : NULL;
  /* the error word of the small-table form (its table staged in shared memory) */
  CqlBuffer* eb = ok ? pooled("jp_error", 16, CQLCUDA_BUFFER_READ_WRITE) : NULL;
  uint32_t stage_error = 0;
  CqlKernel* k = ok ? kernel("join_probe_native") : NULL;
  uint32_t* hc = ok ? (uint32_t*)malloc(D * 4) : NULL;
  uint32_t* hn = ok ? (uint32_t*)malloc(D * core_count * 4) : NULL;
  uint32_t* hx = ok ? (uint32_t*)malloc(D * core_count * 4) : NULL;
  ok = ok && kb && rb && bb && cb && sb && nb && xb && eb && k && hc && hn && hx;
  if (ok)
  {
    uint64_t widths = fk->width == 4 ? 0 : fk->width;
    uint32_t bases[4] = { 0, 0, 0, 0 };
    for (uint32_t i = 0; i < arg_count; i++)
    {
      widths |= (uint64_t)(arg_columns[i]->width == 4 ? 0 : arg_columns[i]->width) << (4 + 4 * i);
      bases[i] = arg_columns[i]->base;
    }
    cqlcuda_kernel_set_arg_buffer(k, 0, fk->buffer);
    for (uint32_t i = 0; i < 4; i++) cqlcuda_kernel_set_arg_buffer(k, 1 + i, i < arg_count ? arg_columns[i]->buffer : fk->buffer);
    cqlcuda_kernel_set_arg_buffer(k, 5, kb);
    cqlcuda_kernel_set_arg_buffer(k, 6, rb);
    cqlcuda_kernel_set_arg_buffer(k, 7, cb);
    cqlcuda_kernel_set_arg_buffer(k, 8, sb);
    cqlcuda_kernel_set_arg_buffer(k, 9, nb);
    cqlcuda_kernel_set_arg_buffer(k, 10, xb);
    cqlcuda_kernel_set_arg_buffer(k, 11, bb);
    cqlcuda_kernel_set_arg_buffer(k, 12, eb);
    cqlcuda_kernel_set_arg_u64(k, 0, rows | (widths << 32));
    cqlcuda_kernel_set_arg_u64(k, 1, core_count | ((uint64_t)bases[0] << 32));
    cqlcuda_kernel_set_arg_u64(k, 2, func_codes | ((uint64_t)bases[1] << 32));
    cqlcuda_kernel_set_arg_u64(k, 3, arg_index_codes | ((uint64_t)arg_signed_bits << 32));
    cqlcuda_kernel_set_arg_u64(k, 4, (size - 1) | ((uint64_t)bases[2] << 32));
    cqlcuda_kernel_set_arg_u64(k, 5, (uint64_t)fk->base | ((uint64_t)bases[3] << 32));
    cqlcuda_kernel_set_arg_u64(k, 6, log2_size | ((uint64_t)bloom_log2 << 32));
    CqlBatch* b = cqlcuda_batch_begin(size * 8, D * (4 + core_count * 16));
    cqlcuda_batch_buffer_write(b, kb, tkeys, size * 4);
    cqlcuda_batch_buffer_write(b, rb, trows, size * 4);
    cqlcuda_batch_buffer_write(b, bb, bloom, (1ull << bloom_log2) * 4);
    cqlcuda_batch_buffer_zero(b, cb, D * 4);
    cqlcuda_batch_buffer_zero(b, sb, D * core_count * 8);
    cqlcuda_batch_buffer_fill(b, nb, D * core_count * 4, 0x7fffffffu);
    cqlcuda_batch_buffer_fill(b, xb, D * core_count * 4, 0x80000000u);
    cqlcuda_batch_buffer_zero(b, eb, 16);
    cqlcuda_batch_kernel_execute(b, k, (uint32_t)((rows + 8191) / 8192 * 256), QE_GPU_WORKGROUP_SIZE);
    cqlcuda_batch_buffer_read(b, cb, hc, D * 4);
    cqlcuda_batch_buffer_read(b, sb, sums, D * core_count * 8);
    cqlcuda_batch_buffer_read(b, nb, hn, D * core_count * 4);
    cqlcuda_batch_buffer_read(b, xb, hx, D * core_count * 4);
    cqlcuda_batch_buffer_read(b, eb, &stage_error, 4);
    ok = cqlcuda_batch_end(b);
    if (ok && stage_error) ok = refuse("the join table's staging into shared memory did not complete");
  }
  if (ok)
  {
    for (uint64_t r = 0; r < D; r++)
    {
      counts[r] = hc[r];
      for (uint32_t e = 0; e < core_count; e++)
      {
        mins[r * core_count + e] = (int32_t)hn[r * core_count + e];
        maxs[r * core_count + e] = (int32_t)hx[r * core_count + e];
      }
    }
  }
  free(tkeys);
  free(trows);
  free(bloom);
  free(hc);
  free(hn);
  free(hx);
  return ok;
}

/* ---- the dim-row pass: groups of the kept dim rows and their accumulators ---- */

/* one aggregate of one group */
typedef struct
{
  uint64_t count;
  double sum, mn, mx;
  int seen;
} JoinAcc;

/* FNV-style hash of a dim row's group values (their f64 bits) */
static uint64_t group_hash(const CqlJoinAgg* q, uint64_t dim_row)
{
  uint64_t h = 1469598103934665603ull;
  for (uint32_t c = 0; c < q->group_count; c++)
  {
    uint64_t bits;
    memcpy(&bits, &q->dim_group_values[c][dim_row], 8);
    h = (h ^ bits) * 1099511628211ull;
    h ^= h >> 29;
  }
  return h;
}

/* two dim rows are in one group when every group value compares equal */
static int same_group(const CqlJoinAgg* q, uint64_t a, uint64_t b)
{
  for (uint32_t c = 0; c < q->group_count; c++)
    if (!(q->dim_group_values[c][a] == q->dim_group_values[c][b])) return 0;
  return 1;
}

/* groups in the order their first dim row was met, found through an open-addressing table of
   (group + 1), each with expr_count accumulators */
typedef struct
{
  uint32_t* slots;
  uint64_t cap, groups, acc_cap;
  uint64_t* rep;
  JoinAcc* acc;
  uint32_t exprs;
} GroupTable;

static int gt_init(GroupTable* t, uint32_t exprs)
{
  t->cap = 64;
  t->acc_cap = 16;
  t->groups = 0;
  t->exprs = exprs;
  t->slots = (uint32_t*)calloc(t->cap, 4);
  t->rep = (uint64_t*)malloc(t->acc_cap * 8);
  t->acc = (JoinAcc*)calloc(t->acc_cap * exprs, sizeof(JoinAcc));
  return t->slots && t->rep && t->acc;
}

static void gt_free(GroupTable* t)
{
  free(t->slots);
  free(t->rep);
  free(t->acc);
  t->slots = NULL;
  t->rep = NULL;
  t->acc = NULL;
}

/* the group of dim_row, a new one when none matches; -1 when memory runs out */
static int64_t gt_find(GroupTable* t, const CqlJoinAgg* q, uint64_t dim_row)
{
  uint64_t pos = 0;
  if (q->group_count == 0)
  {
    if (t->groups) return 0;
  }
  else
  {
    pos = group_hash(q, dim_row) & (t->cap - 1);
    for (;;)
    {
      uint32_t stored = t->slots[pos];
      if (!stored) break;
      if (same_group(q, t->rep[stored - 1], dim_row)) return stored - 1;
      pos = (pos + 1) & (t->cap - 1);
    }
  }
  if (t->groups == t->acc_cap)
  {
    JoinAcc* a2 = (JoinAcc*)realloc(t->acc, t->acc_cap * 2 * t->exprs * sizeof(JoinAcc));
    if (a2) t->acc = a2;
    uint64_t* r2 = a2 ? (uint64_t*)realloc(t->rep, t->acc_cap * 2 * 8) : NULL;
    if (r2) t->rep = r2;
    if (!a2 || !r2) return -1;
    memset(t->acc + t->acc_cap * t->exprs, 0, t->acc_cap * t->exprs * sizeof(JoinAcc));
    t->acc_cap *= 2;
  }
  uint64_t g = t->groups++;
  t->rep[g] = dim_row;
  if (q->group_count == 0) return 0;
  if (t->groups * 2 > t->cap)
  {
    uint32_t* s2 = (uint32_t*)calloc(t->cap * 2, 4);
    if (!s2) return -1;
    free(t->slots);
    t->slots = s2;
    t->cap *= 2;
    for (uint64_t gg = 0; gg < t->groups; gg++)
    {
      uint64_t p2 = group_hash(q, t->rep[gg]) & (t->cap - 1);
      while (t->slots[p2]) p2 = (p2 + 1) & (t->cap - 1);
      t->slots[p2] = (uint32_t)gg + 1;
    }
  }
  else
    t->slots[pos] = (uint32_t)g + 1;
  return (int64_t)g;
}

/* The dim-row pass in two parallel steps: slices of dim rows find their kept rows (those whose key has
   totals), then equal chunks of the kept rows, in dim-row order, are grouped and accumulated; the chunks'
   groups are merged afterwards in chunk order, so groups keep the order of their first dim row and the
   work does not depend on where in the dim table the kept rows lie. */
#define VISIT_SLICE 32768u
#define GROUP_CHUNK 1024u
typedef struct
{
  const CqlJoinAgg* q;
  int signed_key, by_dim_row;
  int64_t min_key;
  uint64_t total_groups;
  const uint64_t* counts;
  const int64_t* sums;
  const int64_t* mins;
  const int64_t* maxs;
  uint32_t core_count;
  const uint32_t* core_of_expr;
  uint64_t visits;
  uint32_t slices;
  uint32_t* kept;          /* each slice's kept dim rows from the slice's start */
  uint64_t* kept_count;    /* per slice */
  uint64_t* kept_before;   /* kept rows of the slices before it */
  uint64_t kept_total;
  uint32_t chunks;
  GroupTable* chunk_groups;
  int* failed;
} VisitCtx;

static uint64_t key_id(const VisitCtx* c, uint64_t dim_row)
{
  uint32_t kw = c->q->dim_keys[dim_row];
  int64_t key_value = c->signed_key ? (int64_t)(int32_t)kw : (int64_t)kw;
  return c->by_dim_row ? dim_row : (uint64_t)(key_value - c->min_key);
}

/* a kept dim row's contribution: its key's totals, or its own value times the key's matches */
static void accumulate(const VisitCtx* c, JoinAcc* a, uint64_t dim_row, uint64_t id)
{
  const CqlJoinAgg* q = c->q;
  uint64_t matches = c->counts[id];
  for (uint32_t e = 0; e < q->expr_count; e++)
  {
    JoinAcc* x = &a[e];
    x->count += matches;
    uint32_t f = q->funcs[e];
    if (f == CQLOPS_FUNC_COUNT) continue;
    double value_sum, value_min, value_max;
    if (q->dim_args && q->dim_args[e])
    {
      double value = q->dim_args[e][dim_row];
      value_sum = value * (double)matches;
      value_min = value_max = value;
    }
    else
    {
      uint64_t slot = id * c->core_count + c->core_of_expr[e];
      value_sum = (double)c->sums[slot];
      value_min = (double)c->mins[slot];
      value_max = (double)c->maxs[slot];
    }
    x->sum += value_sum;
    x->mn = x->seen ? (value_min < x->mn ? value_min : x->mn) : value_min;
    x->mx = x->seen ? (value_max > x->mx ? value_max : x->mx) : value_max;
    x->seen = 1;
  }
}

static void scan_task(void* p, uint32_t task)
{
  VisitCtx* c = (VisitCtx*)p;
  uint64_t v0 = (uint64_t)task * VISIT_SLICE;
  uint64_t v1 = v0 + VISIT_SLICE < c->visits ? v0 + VISIT_SLICE : c->visits;
  const uint64_t* dim_rows = c->q->dim_rows;
  uint32_t* out = c->kept + v0;
  uint64_t n = 0;
  for (uint64_t v = v0; v < v1; v++)
  {
    uint64_t dim_row = dim_rows ? dim_rows[v] : v;
    uint64_t id = key_id(c, dim_row);
    /* written only when kept: a dim table much wider than the fact key's range touches little memory */
    if (id < c->total_groups && c->counts[id] != 0) out[n++] = (uint32_t)dim_row;
  }
  c->kept_count[task] = n;
}

static void group_task(void* p, uint32_t chunk)
{
  VisitCtx* c = (VisitCtx*)p;
  GroupTable* t = &c->chunk_groups[chunk];
  if (!gt_init(t, c->q->expr_count))
  {
    c->failed[chunk] = 1;
    return;
  }
  uint64_t k0 = (uint64_t)chunk * GROUP_CHUNK;
  uint64_t k1 = k0 + GROUP_CHUNK < c->kept_total ? k0 + GROUP_CHUNK : c->kept_total;
  /* the slice holding kept row k0 */
  uint32_t lo = 0, hi = c->slices;
  while (hi - lo > 1)
  {
    uint32_t mid = (lo + hi) / 2;
    if (c->kept_before[mid] <= k0) lo = mid;
    else hi = mid;
  }
  uint32_t slice = lo;
  for (uint64_t k = k0; k < k1; k++)
  {
    while (k >= c->kept_before[slice] + c->kept_count[slice]) slice++;
    uint64_t dim_row = c->kept[(uint64_t)slice * VISIT_SLICE + (k - c->kept_before[slice])];
    int64_t g = gt_find(t, c->q, dim_row);
    if (g < 0)
    {
      c->failed[chunk] = 1;
      return;
    }
    accumulate(c, &t->acc[(uint64_t)g * t->exprs], dim_row, key_id(c, dim_row));
  }
}

static __thread uint32_t* tl_kept = NULL;
static __thread uint64_t tl_kept_cap = 0;

/* ---- strategy 3: a lookup table over the fact key's range ----
   With unique dim keys and one whole-number GROUP BY value of small range (or none), every fact key value
   maps to at most one group: the device builds that table from the dim rows, turns the fact keys into
   group ids (cql_join_lut_map) and the dense group-by aggregates them; the first kept dim row of every
   group comes from the device as well. The host passes over the visited dim rows once (their group
   values' range) and never over the fact rows. Gives way (-1) when the dim keys repeat, the group values
   are not small whole numbers, there are dim-side aggregates or the key range passes 2^24. */
#define LUT_MAX_RANGE (1ull << 24)
#define LUT_MAX_GROUPS 65535u

typedef struct
{
  uint32_t first, gid;
} LutGroup;

static int lut_group_by_first(const void* a, const void* b)
{
  uint32_t x = ((const LutGroup*)a)->first, y = ((const LutGroup*)b)->first;
  return x < y ? -1 : (x > y);
}

static int lut_join_aggregate(const CqlJoinAgg* q, uint32_t core_count, const uint32_t* core_funcs, const CqlColumn* const* core_cols,
                              const uint32_t* core_of_expr, uint64_t max_groups, uint64_t* out_groups, uint64_t* out_group_dim_row,
                              double* out_results)
{
  const CqlColumn* fk = q->fact_key;
  if (!fk->has_range || !fk->buffer || fk->width != 0 || q->group_count > 1) return -1;
  for (uint32_t e = 0; q->dim_args && e < q->expr_count; e++)
    if (q->dim_args[e]) return -1;
  double span = fk->zone_max - fk->zone_min;
  if (!(span >= 0.0) || span + 1.0 > (double)LUT_MAX_RANGE) return -1;
  uint64_t range = (uint64_t)span + 1;
  uint32_t min_bits = (uint32_t)(int64_t)fk->zone_min;
  uint64_t visits = q->dim_rows ? q->dim_count : q->dim_table_rows;
  uint64_t D = q->dim_table_rows;
  if (visits == 0 || D == 0 || D >= 0xffffffffull || visits >= 0xffffffffull) return -1;
  /* device copies of the dim table's key and group columns, when the caller has them resident: nothing is
     uploaded, and the group values' range is the column's zone (a superset of the visited rows' range, which
     only adds empty group ids) */
  const CqlColumn* dkc = q->dim_key_column;
  const CqlColumn* dgc = q->group_count ? q->dim_group_column : NULL;
  int dev_keys = dkc && dkc->buffer && dkc->width == 0 && dkc->rows == D && (dkc->type == CQLOPS_TYPE_U32 || dkc->type == CQLOPS_TYPE_I32);
  int dev_groups = dev_keys && dgc && dgc->buffer && dgc->width == 0 && dgc->rows == D && dgc->has_range &&
                   (dgc->type == CQLOPS_TYPE_U32 || dgc->type == CQLOPS_TYPE_I32);
  /* the group values of the visited rows: whole numbers within LUT_MAX_GROUPS of each other */
  const double* gv = q->group_count ? q->dim_group_values[0] : NULL;
  double vmin = 0.0, vmax = 0.0;
  if (gv && dev_groups)
  {
    vmin = dgc->zone_min;
    vmax = dgc->zone_max;
    if (vmax - vmin > (double)(LUT_MAX_GROUPS - 1)) return -1;
  }
  else if (gv)
  {
    vmin = HUGE_VAL;
    vmax = -HUGE_VAL;
    for (uint64_t v = 0; v < visits; v++)
    {
      uint64_t row = q->dim_rows ? q->dim_rows[v] : v;
      if (row >= D) return -1;
      double x = gv[row];
      if (!(x == (double)(int64_t)x) || x > 9.0e15 || x < -9.0e15) return -1;
      if (x < vmin) vmin = x;
      if (x > vmax) vmax = x;
    }
    if (vmax - vmin > (double)(LUT_MAX_GROUPS - 1)) return -1;
  }
  uint32_t ngroups = gv ? (uint32_t)(vmax - vmin) + 1u : 1u;
  uint64_t rows = fk->rows;
  uint32_t* visit_list = NULL;
  if (q->dim_rows)
  {
    visit_list = (uint32_t*)malloc(visits * 4);
    if (!visit_list) return refuse("out of host memory");
    for (uint64_t v = 0; v < visits; v++)
    {
      if (q->dim_rows[v] >= D)
      {
        free(visit_list);
        return -1;
      }
      visit_list[v] = (uint32_t)q->dim_rows[v];
    }
  }
  CqlBuffer* vbuf = pooled("join_lut_visits", visit_list ? visits * 4 : 4, CQLCUDA_BUFFER_WRITE);
  CqlBuffer* kbuf = dev_keys ? dkc->buffer : pooled("join_lut_dim_keys", D * 4, CQLCUDA_BUFFER_WRITE);
  CqlBuffer* gbuf = dev_groups ? dgc->buffer : pooled("join_lut_group_values", gv ? D * 8 : 8, CQLCUDA_BUFFER_WRITE);
  CqlBuffer* table = pooled("join_lut_table", range * 4, CQLCUDA_BUFFER_READ_WRITE);
  CqlBuffer* visit_of = pooled("join_lut_visit_of", range * 4, CQLCUDA_BUFFER_READ_WRITE);
  CqlBuffer* err = pooled("join_lut_error", 4, CQLCUDA_BUFFER_READ_WRITE);
  CqlBuffer* ids = pooled("join_lut_group_ids", rows * 4, CQLCUDA_BUFFER_READ_WRITE);
  CqlBuffer* present = pooled("join_lut_present", ((range + 31) / 32) * 4, CQLCUDA_BUFFER_READ_WRITE);
  CqlBuffer* first = pooled("join_lut_first", (uint64_t)ngroups * 4, CQLCUDA_BUFFER_READ_WRITE);
  CqlKernel* kb = kernel("cql_join_lut_build");
  CqlKernel* km = kernel("cql_join_lut_map");
  CqlKernel* kf = kernel("cql_join_lut_first");
  uint32_t* h_first = (uint32_t*)malloc((uint64_t)ngroups * 4);
  if (!vbuf || !kbuf || !gbuf || !table || !visit_of || !err || !ids || !present || !first || !kb || !km || !kf || !h_first)
  {
    free(visit_list);
    free(h_first);
    return 0;
  }
  uint64_t group_min_bits;
  memcpy(&group_min_bits, &vmin, 8);
  cqlcuda_kernel_set_arg_buffer(kb, 0, vbuf);
  cqlcuda_kernel_set_arg_buffer(kb, 1, kbuf);
  cqlcuda_kernel_set_arg_buffer(kb, 2, gbuf);
  cqlcuda_kernel_set_arg_buffer(kb, 3, table);
  cqlcuda_kernel_set_arg_buffer(kb, 4, visit_of);
  cqlcuda_kernel_set_arg_buffer(kb, 5, err);
  cqlcuda_kernel_set_arg_u64(kb, 0, visits);
  cqlcuda_kernel_set_arg_u64(kb, 1, visit_list ? 1 : 0);
  cqlcuda_kernel_set_arg_u64(kb, 2, min_bits);
  cqlcuda_kernel_set_arg_u64(kb, 3, range);
  cqlcuda_kernel_set_arg_u64(kb, 4, group_min_bits);
  cqlcuda_kernel_set_arg_u64(kb, 5, gv ? 1 : 0);
  cqlcuda_kernel_set_arg_u64(kb, 6, dev_groups ? dgc->type : CQLOPS_TYPE_F64);   /* the group values' type */
  cqlcuda_kernel_set_arg_buffer(km, 0, fk->buffer);
  cqlcuda_kernel_set_arg_buffer(km, 1, table);
  cqlcuda_kernel_set_arg_buffer(km, 2, ids);
  cqlcuda_kernel_set_arg_buffer(km, 3, present);
  cqlcuda_kernel_set_arg_u64(km, 0, rows);
  cqlcuda_kernel_set_arg_u64(km, 2, min_bits);
  cqlcuda_kernel_set_arg_u64(km, 3, range);
  cqlcuda_kernel_set_arg_u64(km, 4, ngroups);
  cqlcuda_kernel_set_arg_buffer(kf, 0, present);
  cqlcuda_kernel_set_arg_buffer(kf, 1, table);
  cqlcuda_kernel_set_arg_buffer(kf, 2, visit_of);
  cqlcuda_kernel_set_arg_buffer(kf, 3, first);
  cqlcuda_kernel_set_arg_u64(kf, 3, range);
  uint32_t error = 0;
  CqlBatch* b = cqlcuda_batch_begin((visit_list ? visits * 4 : 0) + D * 4 + (gv ? D * 8 : 0), 4 + (uint64_t)ngroups * 4);
  if (visit_list) cqlcuda_batch_buffer_write(b, vbuf, visit_list, visits * 4);
  if (!dev_keys) cqlcuda_batch_buffer_write(b, kbuf, q->dim_keys, D * 4);
  if (gv && !dev_groups) cqlcuda_batch_buffer_write(b, gbuf, gv, D * 8);
  cqlcuda_batch_buffer_fill(b, table, range * 4, 0xffffffffu);
  cqlcuda_batch_buffer_fill(b, first, (uint64_t)ngroups * 4, 0xffffffffu);
  cqlcuda_batch_buffer_zero(b, present, ((range + 31) / 32) * 4);
  cqlcuda_batch_buffer_zero(b, err, 4);
  cqlcuda_batch_kernel_execute(b, kb, (uint32_t)visits, QE_GPU_WORKGROUP_SIZE);
  cqlcuda_batch_kernel_execute(b, km, (uint32_t)(rows < 0xffffffffull ? rows : 0xffffffffull), QE_GPU_WORKGROUP_SIZE);
  cqlcuda_batch_kernel_execute(b, kf, (uint32_t)range, QE_GPU_WORKGROUP_SIZE);
  cqlcuda_batch_buffer_read(b, err, &error, 4);
  cqlcuda_batch_buffer_read(b, first, h_first, (uint64_t)ngroups * 4);
  int ok = cqlcuda_batch_end(b);
  free(visit_list);
  if (ok && error)
  {
    free(h_first);
    return -1;   /* a dim key repeats */
  }
  /* the aggregates per group id (the last id collects the fact rows that join nothing) */
  CqlColumn idcol;
  memset(&idcol, 0, sizeof(idcol));
  idcol.type = CQLOPS_TYPE_U32;
  idcol.rows = rows;
  idcol.buffer = ids;
  idcol.has_range = 1;
  idcol.zone_min = 0.0;
  idcol.zone_max = (double)ngroups;
  uint64_t slots = (uint64_t)ngroups + 1;
  uint64_t* counts = (uint64_t*)malloc(slots * 8);
  int64_t* sums = (int64_t*)malloc(slots * core_count * 8);
  int64_t* mins = (int64_t*)malloc(slots * core_count * 8);
  int64_t* maxs = (int64_t*)malloc(slots * core_count * 8);
  LutGroup* order = (LutGroup*)malloc((uint64_t)ngroups * sizeof(LutGroup));
  uint64_t got_groups = 0;
  int64_t got_min = 0;
  ok = ok && counts && sums && mins && maxs && order &&
       cqlops_group_dense(&idcol, rows, core_count, core_funcs, core_cols, slots, &got_groups, &got_min, counts, sums, mins, maxs);
  int result = ok ? 1 : -1;
  if (ok)
  {
    uint64_t groups = 0;
    for (uint32_t gid = 0; gid < ngroups; gid++)
      if (h_first[gid] != 0xffffffffu && gid < got_groups)
      {
        order[groups].first = h_first[gid];
        order[groups].gid = gid;
        groups++;
      }
    qsort(order, groups, sizeof(LutGroup), lut_group_by_first);
    if (groups > max_groups) result = refuse("more groups than the output arrays hold");
    for (uint64_t g = 0; result == 1 && g < groups; g++)
    {
      uint32_t gid = order[g].gid;
      uint64_t visit = order[g].first;
      out_group_dim_row[g] = q->dim_rows ? q->dim_rows[visit] : visit;
      for (uint32_t e = 0; e < q->expr_count; e++)
      {
        uint64_t slot = (uint64_t)gid * core_count + core_of_expr[e];
        double count = (double)counts[gid], r;
        switch (q->funcs[e])
        {
          case CQLOPS_FUNC_COUNT: r = count; break;
          case CQLOPS_FUNC_SUM: r = (double)sums[slot]; break;
          case CQLOPS_FUNC_AVG: r = counts[gid] ? (double)sums[slot] / count : 0.0; break;
          case CQLOPS_FUNC_MIN: r = (double)mins[slot]; break;
          default: r = (double)maxs[slot]; break;
        }
        out_results[g * q->expr_count + e] = r;
      }
    }
    if (result == 1) *out_groups = groups;
  }
  free(counts);
  free(sums);
  free(mins);
  free(maxs);
  free(order);
  free(h_first);
  return result;
}

typedef struct
{
  int by_dim_row;          /* totals per dim row (the probe), else per key value from min_key (dense) */
  uint64_t total_groups;
  int64_t min_key;
  uint64_t* counts;
  int64_t *sums, *mins, *maxs;
} JoinTotals;

static void join_totals_free(JoinTotals* t)
{
  free(t->counts);
  free(t->sums);
  free(t->mins);
  free(t->maxs);
  memset(t, 0, sizeof(*t));
}

/* The fact-side totals: dense over the fact key's range (strategy 1, or 0 with a range of at most 65536
   values), else per dim row by probing a table of the dim keys (:8607-8617) */
static int join_totals(const CqlJoinAgg* q, uint32_t core_count, const uint32_t* core_funcs, const CqlColumn* const* core_cols, JoinTotals* t)
{
  const CqlColumn* fk = q->fact_key;
  uint64_t rows = fk->rows;
  uint64_t groups_cap = fk->has_range ? (uint64_t)(fk->zone_max - fk->zone_min) + 1 : 0;
  memset(t, 0, sizeof(*t));
  int ok = 0;
  if (q->strategy != 2 && fk->has_range && groups_cap <= 65536)
  {
    t->counts = (uint64_t*)malloc(groups_cap * 8);
    t->sums = (int64_t*)malloc(groups_cap * core_count * 8);
    t->mins = (int64_t*)malloc(groups_cap * core_count * 8);
    t->maxs = (int64_t*)malloc(groups_cap * core_count * 8);
    ok = t->counts && t->sums && t->mins && t->maxs &&
         cqlops_group_dense(fk, rows, core_count, core_funcs, core_cols, groups_cap, &t->total_groups, &t->min_key, t->counts, t->sums, t->mins,
                            t->maxs);
    if (!ok) join_totals_free(t);
  }
  if (!ok)
  {
    if (q->strategy == 1) return refuse("the fact key's range is not small enough for the dense path");
    t->by_dim_row = 1;
    uint64_t D = q->dim_table_rows;
    t->counts = (uint64_t*)malloc(D * 8);
    t->sums = (int64_t*)malloc(D * core_count * 8);
    t->mins = (int64_t*)malloc(D * core_count * 8);
    t->maxs = (int64_t*)malloc(D * core_count * 8);
    ok = t->counts && t->sums && t->mins && t->maxs && probe_totals(q, core_count, core_funcs, core_cols, t->counts, t->sums, t->mins, t->maxs);
    t->total_groups = D;
  }
  if (!ok) join_totals_free(t);
  return ok;
}

/* The dim-row pass over the totals and the outputs (:8619-8776); frees the totals. */
static int join_finish(const CqlJoinAgg* q, JoinTotals* t, const uint32_t* core_of_expr, uint32_t core_count, uint64_t max_groups,
                       uint64_t* out_groups, uint64_t* out_group_dim_row, double* out_results, uint32_t* out_strategy)
{
  const CqlColumn* fk = q->fact_key;
  int ok = 1;
  int by_dim_row = t->by_dim_row;
  uint64_t total_groups = t->total_groups;
  int64_t min_key = t->min_key;
  uint64_t* counts = t->counts;
  int64_t* sums = t->sums;
  int64_t* mins = t->mins;
  int64_t* maxs = t->maxs;
  memset(t, 0, sizeof(*t));
  /* each (filtered) dim row meets its key's totals and joins the group of its group values (:8619-8720);
     the group tables start small and grow with the groups found */
  uint64_t visits = q->dim_rows ? q->dim_count : q->dim_table_rows;
  int signed_key = fk->type == CQLOPS_TYPE_I32;
  VisitCtx vc;
  memset(&vc, 0, sizeof(vc));
  vc.q = q;
  vc.signed_key = signed_key;
  vc.by_dim_row = by_dim_row;
  vc.min_key = min_key;
  vc.total_groups = total_groups;
  vc.counts = counts;
  vc.sums = sums;
  vc.mins = mins;
  vc.maxs = maxs;
  vc.core_count = core_count;
  vc.core_of_expr = core_of_expr;
  vc.visits = visits;
  vc.slices = (uint32_t)((visits + VISIT_SLICE - 1) / VISIT_SLICE);
  /* the kept rows live in a buffer kept per calling thread: a fresh one each call would fault its pages in */
  if (visits + 1 > tl_kept_cap)
  {
    uint32_t* grown = (uint32_t*)realloc(tl_kept, (visits + 1) * sizeof(uint32_t));
    if (grown)
    {
      tl_kept = grown;
      tl_kept_cap = visits + 1;
    }
  }
  vc.kept = visits + 1 <= tl_kept_cap ? tl_kept : NULL;
  vc.kept_count = (uint64_t*)calloc(vc.slices + 1, 8);
  vc.kept_before = (uint64_t*)calloc(vc.slices + 1, 8);
  GroupTable all;
  memset(&all, 0, sizeof(all));
  ok = vc.kept && vc.kept_count && vc.kept_before && gt_init(&all, q->expr_count);
  if (ok) cql_parallel_for(vc.slices, scan_task, &vc);
  for (uint32_t sl = 0; ok && sl < vc.slices; sl++) vc.kept_before[sl + 1] = vc.kept_before[sl] + vc.kept_count[sl];
  vc.kept_total = ok ? vc.kept_before[vc.slices] : 0;
  vc.chunks = (uint32_t)((vc.kept_total + GROUP_CHUNK - 1) / GROUP_CHUNK);
  vc.chunk_groups = (GroupTable*)calloc(vc.chunks ? vc.chunks : 1, sizeof(GroupTable));
  vc.failed = (int*)calloc(vc.chunks ? vc.chunks : 1, sizeof(int));
  ok = ok && vc.chunk_groups && vc.failed;
  if (ok && vc.chunks) cql_parallel_for(vc.chunks, group_task, &vc);
  /* the chunks' groups in chunk order: a group's first dim row decides its place */
  for (uint32_t task = 0; ok && task < vc.chunks; task++)
  {
    const GroupTable* t = &vc.chunk_groups[task];
    if (vc.failed[task])
    {
      ok = 0;
      break;
    }
    for (uint64_t lg = 0; ok && lg < t->groups; lg++)
    {
      int64_t g = gt_find(&all, q, t->rep[lg]);
      if (g < 0)
      {
        ok = 0;
        break;
      }
      for (uint32_t e = 0; e < q->expr_count; e++)
      {
        JoinAcc* x = &all.acc[(uint64_t)g * q->expr_count + e];
        const JoinAcc* y = &t->acc[lg * q->expr_count + e];
        x->count += y->count;
        x->sum += y->sum;
        if (y->seen)
        {
          x->mn = x->seen ? (y->mn < x->mn ? y->mn : x->mn) : y->mn;
          x->mx = x->seen ? (y->mx > x->mx ? y->mx : x->mx) : y->mx;
          x->seen = 1;
        }
      }
    }
  }
  if (vc.chunk_groups)
    for (uint32_t task = 0; task < vc.chunks; task++) gt_free(&vc.chunk_groups[task]);
  free(vc.chunk_groups);
  free(vc.failed);
  free(vc.kept_count);
  free(vc.kept_before);
  uint64_t groups = ok ? all.groups : 0;
  uint64_t* rep = all.rep;
  JoinAcc* acc = all.acc;
  if (ok && groups > max_groups) ok = refuse("more groups than the output arrays hold");
  if (ok)
  {
    for (uint64_t g = 0; g < groups; g++)
    {
      out_group_dim_row[g] = rep[g];
      for (uint32_t e = 0; e < q->expr_count; e++)
      {
        JoinAcc* a = &acc[g * q->expr_count + e];
        double r;
        switch (q->funcs[e])
        {
          case CQLOPS_FUNC_COUNT: r = (double)a->count; break;
          case CQLOPS_FUNC_SUM: r = a->sum; break;
          case CQLOPS_FUNC_AVG: r = a->count ? a->sum / (double)a->count : 0.0; break;
          case CQLOPS_FUNC_MIN: r = a->mn; break;
          default: r = a->mx; break;
        }
        out_results[g * q->expr_count + e] = r;
      }
    }
    *out_groups = groups;
    if (out_strategy) *out_strategy = by_dim_row ? 2u : 1u;
  }
  gt_free(&all);
  free(counts);
  free(sums);
  free(mins);
  free(maxs);
  return ok;
}

/* ---- the dim-row pass on the device, for a dense join over a dim table resident on the device ---- */

typedef struct
{
  uint32_t first, slot;
} SlotFirst;

static int slot_by_first(const void* a, const void* b)
{
  uint32_t x = ((const SlotFirst*)a)->first, y = ((const SlotFirst*)b)->first;
  return x < y ? -1 : (x > y);
}

/* -1 when the query does not take this path (the host pass then runs), else 0 / 1 */
static int join_device_pass(const CqlJoinAgg* q, uint32_t core_count, const uint32_t* core_funcs, const CqlColumn* const* core_cols,
                            const uint32_t* core_of_expr, uint64_t max_groups, uint64_t* out_groups, uint64_t* out_group_dim_row,
                            double* out_results, uint32_t* out_strategy)
{
  const CqlColumn* fk = q->fact_key;
  const CqlColumn* dk = q->dim_key_column;
  const CqlColumn* dg = q->group_count ? q->dim_group_column : NULL;
  if (!dk || !dk->buffer || dk->width != 0 || dk->rows != q->dim_table_rows || !(dk->type == CQLOPS_TYPE_U32 || dk->type == CQLOPS_TYPE_I32))
    return -1;
  if (q->strategy == 2 || !fk->has_range || fk->zone_max - fk->zone_min + 1.0 > 65536.0 || q->group_count > 1) return -1;
  for (uint32_t e = 0; q->dim_args && e < q->expr_count; e++)
    if (q->dim_args[e]) return -1;
  uint64_t slots = 1;
  int64_t group_min = 0;
  if (q->group_count)
  {
    if (!dg || !dg->buffer || dg->width != 0 || dg->rows != q->dim_table_rows || !(dg->type == CQLOPS_TYPE_U32 || dg->type == CQLOPS_TYPE_I32) ||
        !dg->has_range || dg->zone_max - dg->zone_min + 1.0 > 65536.0)
      return -1;
    slots = (uint64_t)(dg->zone_max - dg->zone_min) + 1;
    group_min = (int64_t)dg->zone_min;
  }
  uint64_t visits = q->dim_rows ? q->dim_count : q->dim_table_rows;
  if (visits > 0xffffffffull) return -1;
  CqlDenseTotals t;
  memset(&t, 0, sizeof(t));
  t.keep_open = 1;   /* the dense pass and the dim-row pass in one batch: one wait */
  uint64_t groups_cap = (uint64_t)(fk->zone_max - fk->zone_min) + 1;
  if (!cql_group_dense_device(fk, fk->rows, core_count, core_funcs, core_cols, groups_cap, &t)) return 0;
  uint64_t E = core_count;
  int want_mm = 0;
  for (uint32_t c = 0; c < core_count; c++) want_mm |= core_funcs[c] == CQLOPS_FUNC_MIN || core_funcs[c] == CQLOPS_FUNC_MAX;
  uint64_t counts_at = 0, sums_at = slots * 8, mins_at = sums_at + slots * E * 8, maxs_at = mins_at + slots * E * 4,
           first_at = maxs_at + slots * E * 4, bytes = first_at + slots * 4;
  CqlBuffer* out = pooled("jdim_slots", bytes, CQLCUDA_BUFFER_READ_WRITE);
  CqlBuffer* vb = q->dim_rows ? pooled("jdim_visits", visits * 4, CQLCUDA_BUFFER_WRITE) : NULL;
  CqlKernel* k = kernel("cql_join_dim_fold");
  unsigned char* host = (unsigned char*)malloc(bytes);
  uint32_t* vl = q->dim_rows ? (uint32_t*)malloc(visits * 4) : NULL;
  int ok = out && k && host && (!q->dim_rows || (vb && vl));
  for (uint64_t v = 0; ok && vl && v < visits; v++)
  {
    if (q->dim_rows[v] >= q->dim_table_rows) ok = refuse("a dim row past the dim table");
    else vl[v] = (uint32_t)q->dim_rows[v];
  }
  if (ok)
  {
    cqlcuda_kernel_set_arg_buffer(k, 0, vb ? vb : dk->buffer);
    cqlcuda_kernel_set_arg_buffer(k, 1, dk->buffer);
    cqlcuda_kernel_set_arg_buffer(k, 2, dg ? dg->buffer : dk->buffer);
    cqlcuda_kernel_set_arg_buffer_range(k, 3, t.buffer, 0, t.group_count * 8);
    cqlcuda_kernel_set_arg_buffer_range(k, 4, t.buffer, t.sum_at, t.group_count * E * 8);
    cqlcuda_kernel_set_arg_buffer_range(k, 5, t.buffer, t.min_at, t.group_count * E * 4);
    cqlcuda_kernel_set_arg_buffer_range(k, 6, t.buffer, t.max_at, t.group_count * E * 4);
    cqlcuda_kernel_set_arg_buffer_range(k, 7, out, counts_at, slots * 8);
    cqlcuda_kernel_set_arg_buffer_range(k, 8, out, sums_at, slots * E * 8);
    cqlcuda_kernel_set_arg_buffer_range(k, 9, out, mins_at, slots * E * 4);
    cqlcuda_kernel_set_arg_buffer_range(k, 10, out, maxs_at, slots * E * 4);
    cqlcuda_kernel_set_arg_buffer_range(k, 11, out, first_at, slots * 4);
    /* the kernel reads the low word of each slot (words 0, 2, ..., 14) */
    cqlcuda_kernel_set_arg_u64(k, 0, visits);
    cqlcuda_kernel_set_arg_u64(k, 1, vb ? 1u : 0u);
    cqlcuda_kernel_set_arg_u64(k, 2, (uint32_t)t.min_key);
    cqlcuda_kernel_set_arg_u64(k, 3, t.group_count);
    cqlcuda_kernel_set_arg_u64(k, 4, E);
    cqlcuda_kernel_set_arg_u64(k, 5, (uint32_t)group_min);
    cqlcuda_kernel_set_arg_u64(k, 6, slots);
    cqlcuda_kernel_set_arg_u64(k, 7, (dg ? 1u : 0u) | (want_mm ? 2u : 0u));
    CqlBatch* b = t.batch;
    t.batch = NULL;
    if (vl) cqlcuda_batch_buffer_write(b, vb, vl, visits * 4);
    cqlcuda_batch_buffer_zero(b, out, mins_at);
    cqlcuda_batch_fill_range(b, out, mins_at, slots * E * 4, 0x7fffffffu);
    cqlcuda_batch_fill_range(b, out, maxs_at, slots * E * 4, 0x80000000u);
    cqlcuda_batch_fill_range(b, out, first_at, slots * 4, 0xffffffffu);
    cqlcuda_batch_kernel_execute(b, k, (uint32_t)(visits < 0x7fffff00ull ? visits : 0x7fffff00ull), QE_GPU_WORKGROUP_SIZE);
    cqlcuda_batch_buffer_read(b, out, host, bytes);
    ok = cqlcuda_batch_end(b);
  }
  if (t.batch) cqlcuda_batch_end(t.batch);   /* a refusal above: the dense pass's batch still ends */
  if (ok)
  {
    const uint64_t* counts = (const uint64_t*)(host + counts_at);
    const int64_t* sums = (const int64_t*)(host + sums_at);
    const int32_t* mins = (const int32_t*)(host + mins_at);
    const int32_t* maxs = (const int32_t*)(host + maxs_at);
    const uint32_t* first = (const uint32_t*)(host + first_at);
    SlotFirst* order = (SlotFirst*)malloc(slots * sizeof(SlotFirst));
    uint64_t groups = 0;
    ok = order != NULL;
    for (uint64_t s2 = 0; ok && s2 < slots; s2++)
      if (first[s2] != 0xffffffffu)
      {
        order[groups].first = first[s2];
        order[groups].slot = (uint32_t)s2;
        groups++;
      }
    if (ok && groups > max_groups) ok = refuse("more groups than the output arrays hold");
    if (ok)
    {
      /* groups in the order of their first kept dim row, as the host pass meets them */
      qsort(order, groups, sizeof(SlotFirst), slot_by_first);
      for (uint64_t g = 0; g < groups; g++)
      {
        uint64_t s2 = order[g].slot;
        out_group_dim_row[g] = q->dim_rows ? q->dim_rows[order[g].first] : order[g].first;
        for (uint32_t e = 0; e < q->expr_count; e++)
        {
          uint64_t c = s2 * E + core_of_expr[e];
          double r;
          switch (q->funcs[e])
          {
            case CQLOPS_FUNC_COUNT: r = (double)counts[s2]; break;
            case CQLOPS_FUNC_SUM: r = (double)sums[c]; break;
            case CQLOPS_FUNC_AVG: r = counts[s2] ? (double)sums[c] / (double)counts[s2] : 0.0; break;
            case CQLOPS_FUNC_MIN: r = (double)mins[c]; break;
            default: r = (double)maxs[c]; break;
          }
          out_results[g * q->expr_count + e] = r;
        }
      }
      *out_groups = groups;
      if (out_strategy) *out_strategy = 1u;
    }
    free(order);
  }
  free(host);
  free(vl);
  return ok;
}

/* The fact-side totals each expression needs (:8558-8583): AVG is a SUM and the count, equal
   (function, column) pairs are one total, COUNT-only queries still count */
static int join_core_plan(const CqlJoinAgg* q, uint32_t* core_funcs, const CqlColumn** core_cols, uint32_t* out_core_count,
                          uint32_t* core_of_expr)
{
  uint32_t core_count = 0;
  for (uint32_t e = 0; e < q->expr_count; e++)
  {
    uint32_t f = q->funcs[e];
    if (f > CQLOPS_FUNC_MAX) return refuse("unsupported aggregate function");
    core_of_expr[e] = 0;
    if (f == CQLOPS_FUNC_COUNT || (q->dim_args && q->dim_args[e])) continue;
    uint32_t cf = f == CQLOPS_FUNC_AVG ? CQLOPS_FUNC_SUM : f;
    const CqlColumn* col = q->fact_args[e];
    uint32_t i = 0;
    while (i < core_count && !(core_funcs[i] == cf && core_cols[i] == col)) i++;
    if (i == core_count)
    {
      core_funcs[core_count] = cf;
      core_cols[core_count] = col;
      core_count++;
    }
    core_of_expr[e] = i;
  }
  if (core_count == 0)
  {
    core_funcs[0] = CQLOPS_FUNC_COUNT;
    core_cols[0] = NULL;
    core_count = 1;
  }
  *out_core_count = core_count;
  return 1;
}

int cqlops_join_aggregate(const CqlJoinAgg* q, uint64_t max_groups, uint64_t* out_groups, uint64_t* out_group_dim_row, double* out_results,
                          uint32_t* out_strategy)
{
  cqlops_note_error("");
  const CqlColumn* fk = q->fact_key;
  if (!fk || !(fk->type == CQLOPS_TYPE_U32 || fk->type == CQLOPS_TYPE_I32) || !q->dim_keys || q->expr_count == 0 || q->expr_count > 8)
    return refuse("a U32/I32 fact key, the dim keys and 1 to 8 aggregates");
  if (!cqlops_rows_fit(fk->rows)) return 0;
  for (uint32_t e = 0; e < q->expr_count; e++)
    if (q->fact_args && q->fact_args[e] && !cqlops_rows_fit(q->fact_args[e]->rows)) return 0;
  uint32_t core_funcs[8];
  const CqlColumn* core_cols[8];
  uint32_t core_count = 0, core_of_expr[8];
  if (!join_core_plan(q, core_funcs, core_cols, &core_count, core_of_expr)) return 0;
  if (fk->rows == 0 || (q->dim_rows && q->dim_count == 0) || q->dim_table_rows == 0)
  {
    /* no fact rows, or no dim rows kept: the join has no rows and so no groups (no device work) */
    *out_groups = 0;
    if (out_strategy) *out_strategy = 0;
    return 1;
  }
  /* totals per key: dense over a small key range, else per dim row by probing (:8607-8617) */
  uint64_t groups_cap = fk->has_range ? (uint64_t)(fk->zone_max - fk->zone_min) + 1 : 0;
  /* a mid-sized key range: through a lookup table on the device when the dim side allows it */
  if (q->strategy == 3 || (q->strategy == 0 && fk->has_range && groups_cap > 65536))
  {
    int r = lut_join_aggregate(q, core_count, core_funcs, core_cols, core_of_expr, max_groups, out_groups, out_group_dim_row, out_results);
    if (r >= 0)
    {
      if (r == 1 && out_strategy) *out_strategy = 3u;
      return r;
    }
    if (q->strategy == 3) return refuse("the lookup-table join needs unique dim keys, one small whole-number GROUP BY value and no dim-side aggregates");
    cqlops_note_error("");
  }
  /* a dim table resident on the device: the dim-row pass runs there */
  if (q->dim_key_column)
  {
    int r = join_device_pass(q, core_count, core_funcs, core_cols, core_of_expr, max_groups, out_groups, out_group_dim_row, out_results,
                             out_strategy);
    if (r >= 0) return r;
  }
  JoinTotals totals;
  if (!join_totals(q, core_count, core_funcs, core_cols, &totals)) return 0;
  return join_finish(q, &totals, core_of_expr, core_count, max_groups, out_groups, out_group_dim_row, out_results, out_strategy);
}

/* ---- the fact side streamed through the resident cache (qe_join_probe_stream_core) ---- */

int cqlops_join_aggregate_streamed(CqlResident* r, const CqlJoinAgg* query, const CqlHostColumn* fact_key, const CqlHostColumn* const* fact_args,
                                   uint64_t rows, uint64_t chunk_rows, uint64_t max_groups, uint64_t* out_groups, uint64_t* out_group_dim_row,
                                   double* out_results, uint32_t* out_strategy, uint64_t* out_uploaded_bytes)
{
  cqlops_note_error("");
  if (out_uploaded_bytes) *out_uploaded_bytes = 0;
  if (!r || !query || !fact_key || !(fact_key->type == CQLOPS_TYPE_U32 || fact_key->type == CQLOPS_TYPE_I32) || !fact_key->values ||
      !query->dim_keys || query->expr_count == 0 || query->expr_count > 8)
    return refuse("a U32/I32 host fact key, the dim keys and 1 to 8 aggregates");
  if (query->strategy == 3) return refuse("the lookup-table join does not stream");
  if (!cqlops_rows_fit(rows)) return 0;
  if (chunk_rows == 0) chunk_rows = 1u << 24;
  /* dense over the key's whole range when it is small, else the probe: the same for every chunk */
  uint64_t range = fact_key->has_range ? (uint64_t)(fact_key->zone_max - fact_key->zone_min) + 1 : 0;
  uint32_t strategy = query->strategy ? query->strategy : (fact_key->has_range && range <= 65536 ? 1u : 2u);
  JoinTotals acc;
  memset(&acc, 0, sizeof(acc));
  int have = 0, ok = 1;
  uint32_t core_funcs[8], core_count = 0, core_of_expr[8];
  const CqlColumn* core_cols[8];
  CqlColumn kc;
  CqlJoinAgg qc;
  for (uint64_t start = 0; ok && (start < rows || !have); start += chunk_rows)
  {
    uint64_t n = rows - start < chunk_rows ? rows - start : chunk_rows;
    CqlColumn ac[8];
    const CqlColumn* argp[8] = { NULL };
    CqlBuffer* held[9];
    uint32_t nheld = 0;
    memset(&kc, 0, sizeof(kc));
    if (n > 0)
    {
      /* the chunk's fact columns from the cache; a host column met twice is one device column */
      int hit = 0;
      CqlBuffer* b = (CqlBuffer*)cqlops_resident_acquire(r, fact_key->uid, fact_key->generation, (const char*)fact_key->values + start * 4,
                                                         start, n, 4, &hit);
      if (!b)
      {
        ok = refuse("a chunk could not be held in the cache");
        break;
      }
      if (!hit && out_uploaded_bytes) *out_uploaded_bytes += n * 4;
      held[nheld++] = b;
      kc.buffer = b;
    }
    kc.type = fact_key->type;
    kc.rows = n;
    kc.has_range = fact_key->has_range;
    kc.zone_min = fact_key->zone_min;
    kc.zone_max = fact_key->zone_max;
    for (uint32_t e = 0; ok && e < query->expr_count; e++)
    {
      const CqlHostColumn* h = fact_args ? fact_args[e] : NULL;
      if (!h) continue;
      if (h == fact_key)
      {
        argp[e] = &kc;
        continue;
      }
      uint32_t same = e;
      for (uint32_t j = 0; j < e; j++)
        if (fact_args[j] == h && argp[j]) same = j;
      if (same != e)
      {
        argp[e] = argp[same];
        continue;
      }
      if (!(h->type == CQLOPS_TYPE_U32 || h->type == CQLOPS_TYPE_I32) || !h->values)
      {
        ok = refuse("fact-side aggregates take U32/I32 host columns");
        break;
      }
      memset(&ac[e], 0, sizeof(ac[e]));
      if (n > 0)
      {
        int hit = 0;
        CqlBuffer* b = (CqlBuffer*)cqlops_resident_acquire(r, h->uid, h->generation, (const char*)h->values + start * 4, start, n, 4, &hit);
        if (!b)
        {
          ok = refuse("a chunk could not be held in the cache");
          break;
        }
        if (!hit && out_uploaded_bytes) *out_uploaded_bytes += n * 4;
        held[nheld++] = b;
        ac[e].buffer = b;
      }
      ac[e].type = h->type;
      ac[e].rows = n;
      ac[e].has_range = h->has_range;
      ac[e].zone_min = h->zone_min;
      ac[e].zone_max = h->zone_max;
      argp[e] = &ac[e];
    }
    qc = *query;
    qc.fact_key = &kc;
    qc.fact_args = argp;
    qc.strategy = strategy;
    JoinTotals t;
    memset(&t, 0, sizeof(t));
    if (ok) ok = join_core_plan(&qc, core_funcs, core_cols, &core_count, core_of_expr);
    if (ok && n == 0)
    {
      /* no fact rows: empty totals of the chosen layout */
      t.by_dim_row = strategy == 2;
      t.total_groups = t.by_dim_row ? qc.dim_table_rows : range;
      t.min_key = (int64_t)fact_key->zone_min;
      t.counts = (uint64_t*)calloc(t.total_groups ? t.total_groups : 1, 8);
      t.sums = (int64_t*)calloc((t.total_groups ? t.total_groups : 1) * core_count, 8);
      t.mins = (int64_t*)malloc((t.total_groups ? t.total_groups : 1) * core_count * 8);
      t.maxs = (int64_t*)malloc((t.total_groups ? t.total_groups : 1) * core_count * 8);
      ok = t.counts && t.sums && t.mins && t.maxs;
      for (uint64_t i = 0; ok && i < t.total_groups * core_count; i++)
      {
        t.mins[i] = INT32_MAX;
        t.maxs[i] = INT32_MIN;
      }
      if (!ok) join_totals_free(&t);
    }
    else if (ok)
      ok = join_totals(&qc, core_count, core_funcs, core_cols, &t);
    for (uint32_t i = 0; i < nheld; i++) cqlops_resident_release(r, held[i]);
    if (!ok) break;
    if (!have)
    {
      acc = t;
      have = 1;
      continue;
    }
    if (t.by_dim_row != acc.by_dim_row || t.total_groups != acc.total_groups || t.min_key != acc.min_key)
    {
      join_totals_free(&t);
      ok = refuse("a chunk's totals did not line up with the first chunk's");
      break;
    }
    for (uint64_t g = 0; g < t.total_groups; g++)
    {
      acc.counts[g] += t.counts[g];
      for (uint32_t c = 0; c < core_count; c++)
      {
        uint64_t i = g * core_count + c;
        acc.sums[i] += t.sums[i];
        if (t.mins[i] < acc.mins[i]) acc.mins[i] = t.mins[i];
        if (t.maxs[i] > acc.maxs[i]) acc.maxs[i] = t.maxs[i];
      }
    }
    join_totals_free(&t);
  }
  if (!ok)
  {
    join_totals_free(&acc);
    return 0;
  }
  /* the dim-row pass once, over the chunks' totals */
  qc.fact_args = NULL;
  return join_finish(&qc, &acc, core_of_expr, core_count, max_groups, out_groups, out_group_dim_row, out_results, out_strategy);
}
