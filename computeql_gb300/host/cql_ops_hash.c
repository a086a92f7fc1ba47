/*
 * cql_ops_hash.c - hash GROUP BY with COUNT/SUM/AVG/MIN/MAX, APPROX_COUNT_DISTINCT (HyperLogLog) and
 * APPROX_PERCENTILE (t-digest), driven through the cqlcuda C ABI the way the reference's
 * qe_aggregate_impl drives its GPU (src/query_exec/query_exec.c:10258-12300):
 *
 *   1. keys and arguments as dense f64 (numeric) or raw bytes + offsets (strings)      :10454-10690
 *   2. aggregate_assign into buckets x K slots, buckets grown on overflow and retried   :10792-11243
 *   3. aggregate_compact: occupied slots to dense group ids                             :11251-11330
 *   4a. whole-number arguments: aggregate_hash_reduce_fixed, per-row atomics            :11611-11790
 *   4b. otherwise: csr_scatter into member lists, aggregate_reduce per 4096-row chunk,
 *       HyperLogLog registers and t-digest centroids, folded on the host in chunk order :11826-12275
 *   5. qe_hll_estimate_cardinality (:6711-6737, rounded :12230) and
 *      qe_tdigest_estimate_percentile (:6748-6790)
 */
#include "cqlops.h"

#include <math.h>
#include <stdio.h>
#include <stdlib.h>
#include <string.h>

#define QE_GPU_WORKGROUP_SIZE 256
#define EMPTY 0xffffffffu
#define AGG_ROWS_PER_CHUNK 4096
#define HLL_PRECISION 10
#define HLL_SKETCH_MAX_BYTES (64ull << 20)

void cqlops_note_error(const char* why);

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

/* qe_hll_estimate_cardinality (query_exec.c:6711-6737) */
double cqlops_hll_estimate(const uint32_t* registers, uint64_t m_count)
{
  double m = (double)m_count;
  double alpha = m_count == 16 ? 0.673 : m_count == 32 ? 0.697 : m_count == 64 ? 0.709 : 0.7213 / (1.0 + 1.079 / m);
  double sum = 0.0;
  uint64_t zeros = 0;
  for (uint64_t i = 0; i < m_count; i++)
  {
    sum += 1.0 / (double)((uint64_t)1 << registers[i]);
    if (registers[i] == 0) zeros++;
  }
  double estimate = alpha * m * m / sum;
  if (estimate <= 2.5 * m && zeros > 0) estimate = m * log(m / (double)zeros);
  return estimate;
}

typedef struct
{
  float mean;
  float weight;
} Centroid;

static int centroid_cmp(const void* a, const void* b)
{
  float x = ((const Centroid*)a)->mean, y = ((const Centroid*)b)->mean;
  return (x > y) - (x < y);
}

/* qe_tdigest_estimate_percentile (query_exec.c:6748-6790) */
double cqlops_tdigest_percentile(float* means, float* weights, uint64_t count, double fraction)
{
  if (count == 0) return 0.0;
  Centroid* c = (Centroid*)malloc(sizeof(Centroid) * count);
  if (!c) return 0.0;
  for (uint64_t i = 0; i < count; i++)
  {
    c[i].mean = means[i];
    c[i].weight = weights[i];
  }
  qsort(c, count, sizeof(Centroid), centroid_cmp);
  double total = 0.0;
  for (uint64_t i = 0; i < count; i++) total += c[i].weight;
  double result;
  if (total <= 0.0) result = 0.0;
  else
  {
    double target = fraction * total, cumulative = 0.0, prev_pos = -1.0, prev_mean = (double)c[0].mean;
    result = (double)c[count - 1].mean;
    for (uint64_t i = 0; i < count; i++)
    {
      double pos = cumulative + (double)c[i].weight * 0.5;
      if (target <= pos)
      {
        if (prev_pos < 0.0) result = (double)c[i].mean;
        else
        {
          double t = (target - prev_pos) / (pos - prev_pos);
          result = prev_mean + t * ((double)c[i].mean - prev_mean);
        }
        break;
      }
      cumulative += c[i].weight;
      prev_pos = pos;
      prev_mean = (double)c[i].mean;
    }
  }
  free(c);
  return result;
}

/* a numeric device column widened to a dense f64 buffer */
static CqlBuffer* widen(const CqlColumn* col, const char* name)
{
  if (col->width != 0 || !col->buffer) return NULL;
  CqlBuffer* out = pooled(name, col->rows * 8, CQLCUDA_BUFFER_READ_WRITE);
  CqlKernel* k = kernel("cql_widen_f64");
  if (!out || !k) return NULL;
  cqlcuda_kernel_set_arg_buffer(k, 0, col->buffer);
  cqlcuda_kernel_set_arg_buffer(k, 1, out);
  cqlcuda_kernel_set_arg_u64(k, 0, col->rows);
  cqlcuda_kernel_set_arg_u64(k, 1, col->type);
  CqlBatch* b = cqlcuda_batch_begin(0, 0);
  cqlcuda_batch_kernel_execute(b, k, (uint32_t)(col->rows < 0xffffffffull ? col->rows : 0xffffffffull), QE_GPU_WORKGROUP_SIZE);
  return cqlcuda_batch_end(b) ? out : NULL;
}

static int whole_number_arg(const CqlColumn* col)
{
  return (col->type == CQLOPS_TYPE_U32 || col->type == CQLOPS_TYPE_I32) && col->has_range && col->zone_min >= -2147483648.0 &&
         col->zone_max <= 2147483647.0;
}

int cqlops_group_hash(const CqlColumn* keys, uint32_t key_count, uint32_t expr_count, const uint32_t* funcs, const CqlColumn* const* args,
                      const double* params, uint64_t group_hint, uint32_t path, uint64_t max_groups, uint64_t* out_group_count,
                      uint64_t* out_repr_row, uint64_t* out_counts, double* out_results, uint32_t* out_path)
{
  cqlops_note_error("");
  if (key_count > 4 || expr_count == 0 || expr_count > 8) return refuse("0 to 4 keys and 1 to 8 aggregates");
  /* no GROUP BY: one bucket of one slot takes every row (:10796-10801) */
  uint64_t rows = key_count ? keys[0].rows : 0;
  for (uint32_t e = 0; e < expr_count && !key_count; e++)
    if (args[e]) rows = args[e]->rows;
  if (rows >= 0xffffffffull) return refuse("row count out of range");
  if (rows == 0)
  {
    /* no rows, no groups: an aggregate over nothing is the caller's empty result */
    *out_group_count = 0;
    if (out_path) *out_path = 0;
    return 1;
  }
  uint32_t string_mask = 0;
  CqlBuffer* key_data[4] = { 0 };
  CqlBuffer* key_off[4] = { 0 };
  char name[64];
  for (uint32_t c = 0; c < key_count; c++)
  {
    if (keys[c].rows != rows) return refuse("keys of different lengths");
    if (keys[c].type == CQLOPS_TYPE_STRING8)
    {
      if (!keys[c].offsets || keys[c].dict) return refuse("a string key is read as raw bytes and offsets");
      string_mask |= 1u << c;
      key_data[c] = keys[c].buffer;
      key_off[c] = keys[c].offsets;
    }
    else
    {
      snprintf(name, sizeof(name), "cqlops_hash_key_f64_%u", c);
      key_data[c] = widen(&keys[c], name);
      if (!key_data[c]) return refuse("a key column could not be widened to f64 (narrow or sequence encodings are not taken here)");
      key_off[c] = key_data[c];
    }
  }
  int has_sketch = 0, all_whole = 1;
  uint32_t func_codes = 0;
  for (uint32_t e = 0; e < expr_count; e++)
  {
    if (funcs[e] > CQLOPS_FUNC_APPROX_PERCENTILE) return refuse("unsupported aggregate function");
    func_codes |= (funcs[e] & 0xfu) << (4 * e);
    if (funcs[e] == CQLOPS_FUNC_APPROX_COUNT_DISTINCT || funcs[e] == CQLOPS_FUNC_APPROX_PERCENTILE) has_sketch = 1;
    if (funcs[e] != CQLOPS_FUNC_COUNT)
    {
      if (!args[e] || args[e]->rows != rows) return refuse("an aggregate needs an argument column of the table's length");
      if (!whole_number_arg(args[e])) all_whole = 0;
    }
  }
  int use_fixed = !has_sketch && all_whole;
  if (path == 1) use_fixed = 0;
  if (path == 2 && (!use_fixed)) return refuse("the fixed-point reduce takes whole-number COUNT/SUM/AVG/MIN/MAX only");
  CqlBuffer* arg_f64[8] = { 0 };
  for (uint32_t e = 0; e < expr_count; e++)
  {
    if (funcs[e] == CQLOPS_FUNC_COUNT) continue;
    snprintf(name, sizeof(name), "cqlops_hash_arg_f64_%u", e);
    arg_f64[e] = widen(args[e], name);
    if (!arg_f64[e]) return refuse("an argument column could not be widened to f64");
  }

  /* buckets: ~64 rows per group unless the caller knows better (:10792-10826) */
  uint64_t max_buckets = 1;
  while (max_buckets < rows) max_buckets <<= 1;
  uint64_t buckets = 16;
  if (key_count == 0)
  {
    buckets = 1;
    max_buckets = 1;
  }
  else if (group_hint > 0)
  {
    uint64_t wanted = group_hint + group_hint / 4;
    while (buckets < wanted && buckets < max_buckets) buckets <<= 1;
  }
  else
    while (buckets < rows / 64 && buckets < max_buckets) buckets <<= 1;
  uint64_t K = key_count ? 8 : 1;
  CqlKernel* assign = kernel("aggregate_assign");
  if (!assign) return 0;
  CqlBuffer *owner = NULL, *count = NULL, *row_slot = NULL, *overflow = NULL;
  uint64_t slots = 0;
  for (int attempt = 0; attempt < 16; attempt++)
  {
    slots = buckets * K;
    owner = pooled("agg_owner_buf", slots * 4, CQLCUDA_BUFFER_READ_WRITE);
    count = pooled("agg_count_buf", slots * 4, CQLCUDA_BUFFER_READ_WRITE);
    row_slot = pooled("agg_row_slot_buf", rows * 4, CQLCUDA_BUFFER_READ_WRITE);
    overflow = pooled("agg_overflow_buf", 4, CQLCUDA_BUFFER_READ_WRITE);
    if (!owner || !count || !row_slot || !overflow) return 0;
    for (uint32_t c = 0; c < 4; c++)
    {
      /* key bindings past the key count are never read: bound to the row-slot buffer */
      cqlcuda_kernel_set_arg_buffer(assign, 4 + 2 * c, c < key_count ? key_data[c] : row_slot);
      cqlcuda_kernel_set_arg_buffer(assign, 5 + 2 * c, c < key_count ? key_off[c] : row_slot);
    }
    cqlcuda_kernel_set_arg_buffer(assign, 0, owner);
    cqlcuda_kernel_set_arg_buffer(assign, 1, count);
    cqlcuda_kernel_set_arg_buffer(assign, 2, row_slot);
    cqlcuda_kernel_set_arg_buffer(assign, 3, overflow);
    cqlcuda_kernel_set_arg_u64(assign, 0, rows);
    cqlcuda_kernel_set_arg_u64(assign, 1, buckets);
    cqlcuda_kernel_set_arg_u64(assign, 2, K);
    cqlcuda_kernel_set_arg_u64(assign, 3, key_count);
    cqlcuda_kernel_set_arg_u64(assign, 4, string_mask);
    uint32_t over = 0;
    CqlBatch* b = cqlcuda_batch_begin(0, 4);
    cqlcuda_batch_buffer_fill(b, owner, slots * 4, EMPTY);
    cqlcuda_batch_buffer_zero(b, count, slots * 4);
    cqlcuda_batch_buffer_fill(b, row_slot, rows * 4, EMPTY);
    cqlcuda_batch_buffer_zero(b, overflow, 4);
    cqlcuda_batch_kernel_execute(b, assign, (uint32_t)rows, QE_GPU_WORKGROUP_SIZE);
    cqlcuda_batch_buffer_read(b, overflow, &over, 4);
    if (!cqlcuda_batch_end(b)) return 0;
    if (over == 0 || key_count == 0) break;
    /* grow the buckets by how badly they missed, then K (:11226-11243) */
    if (buckets < max_buckets)
    {
      double frac = (double)over / (double)rows;
      uint64_t growth = frac >= 0.20 ? 8 : (frac >= 0.05 ? 4 : 2);
      buckets = buckets * growth < max_buckets ? buckets * growth : max_buckets;
    }
    else K *= 2;
    if (attempt == 15) return refuse("the group-by hash table kept overflowing");
  }

  /* compaction: offsets[slot] becomes the dense group id of an occupied slot */
  uint64_t blocks = (slots + 255) / 256;
  uint64_t max_g = slots < rows ? slots : rows;
  CqlBuffer* offsets = pooled("agg_compact_offsets_buf", (slots + 1) * 4, CQLCUDA_BUFFER_READ_WRITE);
  CqlBuffer* block_sums = pooled("agg_compact_block_sum_buf", blocks * 4, CQLCUDA_BUFFER_READ_WRITE);
  CqlBuffer* out_owner = pooled("agg_compact_owner_buf", max_g * 4, CQLCUDA_BUFFER_READ_WRITE);
  CqlBuffer* out_count = pooled("agg_compact_count_buf", max_g * 4, CQLCUDA_BUFFER_READ_WRITE);
  CqlBuffer* total_buf = pooled("agg_compact_total_buf", 4, CQLCUDA_BUFFER_READ_WRITE);
  CqlKernel* compact = kernel("aggregate_compact");
  if (!offsets || !block_sums || !out_owner || !out_count || !total_buf || !compact) return 0;
  cqlcuda_kernel_set_arg_buffer(compact, 0, count);
  cqlcuda_kernel_set_arg_buffer(compact, 1, owner);
  cqlcuda_kernel_set_arg_buffer(compact, 2, offsets);
  cqlcuda_kernel_set_arg_buffer(compact, 3, block_sums);
  cqlcuda_kernel_set_arg_buffer(compact, 4, out_owner);
  cqlcuda_kernel_set_arg_buffer(compact, 5, out_count);
  cqlcuda_kernel_set_arg_buffer(compact, 6, total_buf);
  cqlcuda_kernel_set_arg_u64(compact, 0, slots);
  uint32_t groups32 = 0;
  {
    CqlBatch* b = cqlcuda_batch_begin(0, 4);
    cqlcuda_kernel_set_arg_u64(compact, 1, 0);
    cqlcuda_batch_kernel_execute(b, compact, (uint32_t)(blocks * 256), 256);
    cqlcuda_kernel_set_arg_u64(compact, 1, 1);
    cqlcuda_batch_kernel_execute(b, compact, 256, 256);
    cqlcuda_kernel_set_arg_u64(compact, 1, 2);
    cqlcuda_batch_kernel_execute(b, compact, (uint32_t)(blocks * 256), 256);
    cqlcuda_batch_buffer_read(b, total_buf, &groups32, 4);
    if (!cqlcuda_batch_end(b)) return 0;
  }
  uint64_t groups = groups32;
  if (groups > max_groups) return refuse("more groups than the output arrays hold");
  uint32_t* g_owner = (uint32_t*)malloc((groups ? groups : 1) * 4);
  uint32_t* g_count = (uint32_t*)malloc((groups ? groups : 1) * 4);
  if (!g_owner || !g_count)
  {
    free(g_owner);
    free(g_count);
    return 0;
  }
  {
    CqlBatch* b = cqlcuda_batch_begin(0, groups * 8);
    cqlcuda_batch_buffer_read(b, out_owner, g_owner, groups * 4);
    cqlcuda_batch_buffer_read(b, out_count, g_count, groups * 4);
    if (!cqlcuda_batch_end(b))
    {
      free(g_owner);
      free(g_count);
      return 0;
    }
  }
  for (uint64_t g = 0; g < groups; g++)
  {
    out_repr_row[g] = g_owner[g];
    out_counts[g] = g_count[g];
  }
  int ok = 1;
  if (use_fixed)
  {
    /* 4a: per-row atomics into per-group arrays; the compact offsets are the slot -> group map */
    CqlKernel* hr = kernel("aggregate_hash_reduce_fixed");
    uint64_t cells = groups * expr_count;
    CqlBuffer* sums = pooled("agg_hash_sum_buf", cells * 8, CQLCUDA_BUFFER_READ_WRITE);
    CqlBuffer* cnts = pooled("agg_hash_count_buf", cells * 4, CQLCUDA_BUFFER_READ_WRITE);
    CqlBuffer* mins = pooled("agg_hash_min_buf", cells * 4, CQLCUDA_BUFFER_READ_WRITE);
    CqlBuffer* maxs = pooled("agg_hash_max_buf", cells * 4, CQLCUDA_BUFFER_READ_WRITE);
    int64_t* hs = (int64_t*)malloc(cells * 8 + 8);
    int32_t* hmn = (int32_t*)malloc(cells * 4 + 4);
    int32_t* hmx = (int32_t*)malloc(cells * 4 + 4);
    ok = hr && sums && cnts && mins && maxs && hs && hmn && hmx;
    if (ok)
    {
      cqlcuda_kernel_set_arg_buffer(hr, 0, row_slot);
      cqlcuda_kernel_set_arg_buffer(hr, 1, offsets);
      cqlcuda_kernel_set_arg_buffer(hr, 2, sums);
      cqlcuda_kernel_set_arg_buffer(hr, 3, cnts);
      cqlcuda_kernel_set_arg_buffer(hr, 4, mins);
      cqlcuda_kernel_set_arg_buffer(hr, 5, maxs);
      for (uint32_t e = 0; e < 8; e++) cqlcuda_kernel_set_arg_buffer(hr, 6 + e, arg_f64[e] ? arg_f64[e] : row_slot);
      cqlcuda_kernel_set_arg_u64(hr, 0, rows);
      cqlcuda_kernel_set_arg_u64(hr, 1, expr_count);
      cqlcuda_kernel_set_arg_u64(hr, 2, func_codes);
      cqlcuda_kernel_set_arg_u64(hr, 3, 0); /* whole numbers: every scale exponent 0 */
      CqlBatch* b = cqlcuda_batch_begin(0, cells * 16);
      cqlcuda_batch_buffer_zero(b, sums, cells * 8);
      cqlcuda_batch_buffer_zero(b, cnts, cells * 4);
      cqlcuda_batch_buffer_fill(b, mins, cells * 4, 0x7fffffffu);
      cqlcuda_batch_buffer_fill(b, maxs, cells * 4, 0x80000000u);
      cqlcuda_batch_kernel_execute(b, hr, (uint32_t)rows, QE_GPU_WORKGROUP_SIZE);
      cqlcuda_batch_buffer_read(b, sums, hs, cells * 8);
      cqlcuda_batch_buffer_read(b, mins, hmn, cells * 4);
      cqlcuda_batch_buffer_read(b, maxs, hmx, cells * 4);
      ok = cqlcuda_batch_end(b);
    }
    if (ok)
    {
      for (uint64_t g = 0; g < groups; g++)
        for (uint32_t e = 0; e < expr_count; e++)
        {
          uint64_t i = g * expr_count + e;
          double r;
          switch (funcs[e])
          {
            case CQLOPS_FUNC_COUNT: r = (double)g_count[g]; break;
            case CQLOPS_FUNC_SUM: r = (double)hs[i]; break;
            case CQLOPS_FUNC_AVG: r = (double)hs[i] / (double)g_count[g]; break;
            case CQLOPS_FUNC_MIN: r = (double)hmn[i]; break;
            default: r = (double)hmx[i]; break;
          }
          out_results[i] = r;
        }
    }
    free(hs);
    free(hmn);
    free(hmx);
  }
  else
  {
    /* 4b: member lists, group g's members at [start[g], start[g] + count[g]) */
    uint32_t* g_start = (uint32_t*)malloc((groups + 1) * 4);
    uint32_t* h_offsets = (uint32_t*)malloc((slots + 1) * 4);
    uint32_t* h_counts = (uint32_t*)malloc(slots * 4);
    uint32_t* cursor = (uint32_t*)malloc(slots * 4);
    ok = g_start && h_offsets && h_counts && cursor;
    if (ok)
    {
      CqlBatch* b = cqlcuda_batch_begin(0, slots * 8);
      cqlcuda_batch_buffer_read(b, offsets, h_offsets, slots * 4);
      cqlcuda_batch_buffer_read(b, count, h_counts, slots * 4);
      ok = cqlcuda_batch_end(b);
    }
    if (ok)
    {
      uint32_t run = 0;
      for (uint64_t g = 0; g < groups; g++)
      {
        g_start[g] = run;
        run += g_count[g];
      }
      g_start[groups] = run;
      for (uint64_t s = 0; s < slots; s++) cursor[s] = h_counts[s] ? g_start[h_offsets[s]] : 0u;
      uint64_t total_chunks = 0;
      for (uint64_t g = 0; g < groups; g++) total_chunks += g_count[g] ? (g_count[g] + AGG_ROWS_PER_CHUNK - 1) / AGG_ROWS_PER_CHUNK : 1;
      uint32_t* chunk_range = (uint32_t*)malloc(total_chunks * 8 + 8);
      uint32_t* chunk_group = (uint32_t*)malloc(total_chunks * 4 + 4);
      uint64_t* chunk_base = (uint64_t*)malloc((groups + 1) * 8);
      uint32_t num_hll = 0, num_pct = 0, hll_slot_packed = 0, pct_slot_packed = 0;
      for (uint32_t e = 0; e < expr_count; e++)
      {
        if (funcs[e] == CQLOPS_FUNC_APPROX_COUNT_DISTINCT) hll_slot_packed |= (num_hll++) << (4 * e);
        if (funcs[e] == CQLOPS_FUNC_APPROX_PERCENTILE) pct_slot_packed |= (num_pct++) << (4 * e);
      }
      uint64_t hll_words = 1ull << HLL_PRECISION;
      uint64_t sketch_bytes = (groups ? groups : 1) * (num_hll ? num_hll : 1) * hll_words * 4;
      uint64_t digest_words = total_chunks * (num_pct ? num_pct : 1) * 256;
      if (num_hll && sketch_bytes > HLL_SKETCH_MAX_BYTES) ok = refuse("the HyperLogLog sketches exceed QE_HLL_SKETCH_MAX_TOTAL_BYTES (64 MB)");
      uint64_t c = 0;
      for (uint64_t g = 0; g < groups && ok; g++)
      {
        uint64_t n = g_count[g] ? (g_count[g] + AGG_ROWS_PER_CHUNK - 1) / AGG_ROWS_PER_CHUNK : 1;
        chunk_base[g] = c;
        for (uint64_t k = 0; k < n; k++, c++)
        {
          uint32_t s = g_start[g] + (uint32_t)(k * AGG_ROWS_PER_CHUNK);
          uint32_t e2 = s + AGG_ROWS_PER_CHUNK < g_start[g] + g_count[g] ? s + AGG_ROWS_PER_CHUNK : g_start[g] + g_count[g];
          chunk_range[c * 2] = s;
          chunk_range[c * 2 + 1] = e2;
          chunk_group[c] = (uint32_t)g;
        }
      }
      CqlBuffer* cursor_buf = pooled("agg_cursor_buf", slots * 4, CQLCUDA_BUFFER_READ_WRITE);
      CqlBuffer* members = pooled("agg_members_buf", rows * 4, CQLCUDA_BUFFER_READ_WRITE);
      CqlBuffer* range_buf = pooled("agg_chunk_range_buf", total_chunks * 8, CQLCUDA_BUFFER_WRITE);
      CqlBuffer* group_buf = pooled("agg_chunk_group_buf", total_chunks * 4, CQLCUDA_BUFFER_WRITE);
      CqlBuffer* repr_buf = pooled("agg_repr_buf", groups * 4, CQLCUDA_BUFFER_READ_WRITE);
      CqlBuffer* partials_buf = pooled("agg_partials_buf", total_chunks * expr_count * 32, CQLCUDA_BUFFER_READ_WRITE);
      CqlBuffer* sketch_buf = pooled("agg_sketch_buf", sketch_bytes, CQLCUDA_BUFFER_READ_WRITE);
      CqlBuffer* dmean_buf = pooled("agg_digest_mean_buf", digest_words * 4, CQLCUDA_BUFFER_READ_WRITE);
      CqlBuffer* dweight_buf = pooled("agg_digest_weight_buf", digest_words * 4, CQLCUDA_BUFFER_READ_WRITE);
      CqlKernel* scatter = kernel("csr_scatter");
      CqlKernel* reduce = kernel("aggregate_reduce");
      double* partials = (double*)malloc(total_chunks * expr_count * 32 + 8);
      uint32_t* sketch = num_hll ? (uint32_t*)malloc(sketch_bytes) : NULL;
      float* dmean = num_pct ? (float*)malloc(digest_words * 4) : NULL;
      float* dweight = num_pct ? (float*)malloc(digest_words * 4) : NULL;
      ok = ok && chunk_range && chunk_group && chunk_base && cursor_buf && members && range_buf && group_buf && repr_buf && partials_buf &&
           sketch_buf && dmean_buf && dweight_buf && scatter && reduce && partials && (!num_hll || sketch) && (!num_pct || (dmean && dweight));
      if (ok)
      {
        cqlcuda_kernel_set_arg_buffer(scatter, 0, row_slot);
        cqlcuda_kernel_set_arg_buffer(scatter, 1, cursor_buf);
        cqlcuda_kernel_set_arg_buffer(scatter, 2, members);
        cqlcuda_kernel_set_arg_u64(scatter, 0, rows);
        cqlcuda_kernel_set_arg_buffer(reduce, 0, members);
        cqlcuda_kernel_set_arg_buffer(reduce, 1, range_buf);
        cqlcuda_kernel_set_arg_buffer(reduce, 2, group_buf);
        cqlcuda_kernel_set_arg_buffer(reduce, 3, repr_buf);
        cqlcuda_kernel_set_arg_buffer(reduce, 4, partials_buf);
        for (uint32_t e = 0; e < 8; e++) cqlcuda_kernel_set_arg_buffer(reduce, 5 + e, arg_f64[e] ? arg_f64[e] : members);
        cqlcuda_kernel_set_arg_buffer(reduce, 13, sketch_buf);
        cqlcuda_kernel_set_arg_buffer(reduce, 14, dmean_buf);
        cqlcuda_kernel_set_arg_buffer(reduce, 15, dweight_buf);
        cqlcuda_kernel_set_arg_u64(reduce, 0, total_chunks);
        cqlcuda_kernel_set_arg_u64(reduce, 1, expr_count);
        cqlcuda_kernel_set_arg_u64(reduce, 2, func_codes);
        cqlcuda_kernel_set_arg_u64(reduce, 3, 0);
        cqlcuda_kernel_set_arg_u64(reduce, 4, HLL_PRECISION);
        cqlcuda_kernel_set_arg_u64(reduce, 5, hll_slot_packed);
        cqlcuda_kernel_set_arg_u64(reduce, 6, num_hll);
        cqlcuda_kernel_set_arg_u64(reduce, 7, num_pct | ((uint64_t)pct_slot_packed << 32));
        CqlBatch* b = cqlcuda_batch_begin(slots * 4 + total_chunks * 12, total_chunks * expr_count * 32 + sketch_bytes + 2 * digest_words * 4);
        cqlcuda_batch_buffer_write(b, cursor_buf, cursor, slots * 4);
        cqlcuda_batch_buffer_write(b, range_buf, chunk_range, total_chunks * 8);
        cqlcuda_batch_buffer_write(b, group_buf, chunk_group, total_chunks * 4);
        if (num_hll) cqlcuda_batch_buffer_zero(b, sketch_buf, sketch_bytes);
        cqlcuda_batch_kernel_execute(b, scatter, (uint32_t)rows, QE_GPU_WORKGROUP_SIZE);
        cqlcuda_batch_kernel_execute(b, reduce, (uint32_t)(total_chunks * QE_GPU_WORKGROUP_SIZE), QE_GPU_WORKGROUP_SIZE);
        cqlcuda_batch_buffer_read(b, partials_buf, partials, total_chunks * expr_count * 32);
        if (num_hll) cqlcuda_batch_buffer_read(b, sketch_buf, sketch, sketch_bytes);
        if (num_pct)
        {
          cqlcuda_batch_buffer_read(b, dmean_buf, dmean, digest_words * 4);
          cqlcuda_batch_buffer_read(b, dweight_buf, dweight, digest_words * 4);
        }
        ok = cqlcuda_batch_end(b);
      }
      if (ok)
      {
        /* fold each group's chunks in chunk order (:12180-12215) */
        float* cm = NULL;
        float* cw = NULL;
        for (uint64_t g = 0; g < groups && ok; g++)
        {
          uint64_t n = g_count[g] ? (g_count[g] + AGG_ROWS_PER_CHUNK - 1) / AGG_ROWS_PER_CHUNK : 1;
          for (uint32_t e = 0; e < expr_count; e++)
          {
            double acc = 0.0, mn = 1.0e300, mx = -1.0e300, cnt = 0.0;
            for (uint64_t k = 0; k < n; k++)
            {
              const double* pp = &partials[((chunk_base[g] + k) * expr_count + e) * 4];
              acc += pp[0];
              cnt += pp[1];
              mn = pp[2] < mn ? pp[2] : mn;
              mx = pp[3] > mx ? pp[3] : mx;
            }
            double r;
            switch (funcs[e])
            {
              case CQLOPS_FUNC_COUNT: r = cnt; break;
              case CQLOPS_FUNC_SUM: r = acc; break;
              case CQLOPS_FUNC_AVG: r = cnt > 0 ? acc / cnt : 0.0; break;
              case CQLOPS_FUNC_MIN: r = mn; break;
              case CQLOPS_FUNC_MAX: r = mx; break;
              case CQLOPS_FUNC_APPROX_COUNT_DISTINCT:
                r = round(cqlops_hll_estimate(&sketch[(g * num_hll + ((hll_slot_packed >> (4 * e)) & 0xfu)) * hll_words], hll_words));
                break;
              default:
              {
                uint64_t cap = n * 256, v = 0;
                cm = (float*)realloc(cm, cap * 4);
                cw = (float*)realloc(cw, cap * 4);
                if (!cm || !cw)
                {
                  ok = 0;
                  r = 0.0;
                  break;
                }
                uint32_t ps = (pct_slot_packed >> (4 * e)) & 0xfu;
                for (uint64_t k = 0; k < n; k++)
                {
                  uint64_t base = ((chunk_base[g] + k) * num_pct + ps) * 256;
                  for (uint32_t t = 0; t < 256; t++)
                    if (dweight[base + t] > 0.0f)
                    {
                      cm[v] = dmean[base + t];
                      cw[v] = dweight[base + t];
                      v++;
                    }
                }
                r = cqlops_tdigest_percentile(cm, cw, v, params ? params[e] : 0.5);
              }
            }
            out_results[g * expr_count + e] = r;
          }
        }
        free(cm);
        free(cw);
      }
      free(chunk_range);
      free(chunk_group);
      free(chunk_base);
      free(partials);
      free(sketch);
      free(dmean);
      free(dweight);
    }
    free(g_start);
    free(h_offsets);
    free(h_counts);
    free(cursor);
  }
  free(g_owner);
  free(g_count);
  if (ok)
  {
    *out_group_count = groups;
    if (out_path) *out_path = use_fixed ? 2u : 1u;
  }
  return ok;
}
